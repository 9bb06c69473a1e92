"""Mode-resolved transmission of the electron (tight-binding) branch:
pf_transport_tdb_modes_ex_dev with PF_MODES_ELECTRON (the normalisation of
tb/velocity_mat.f90: V = U^H Gamma U, t = i V^1/2 U^-1 G U^-H V^1/2).

On a clean single-orbital ribbon (no transverse folding: one unfolding
label) the mode sums must add up to the Caroli transmission of the same
call at energies of both signs, the pristine ribbon's T must be the
integer number of open channels, and for E > 0 the electron and phonon
normalisations must give the same sums (their scalings cancel in t, r)."""
import numpy as np
import pytest

from phinfortran_gb300 import systems as S
from phinfortran_gb300.modes import SUM_NAMES, transport_tdb_modes

pytestmark = pytest.mark.gpu


class RibbonLeads:
    """Lead geometry of a ribbon without transverse images: one label."""

    def __init__(self, n):
        self.n = n
        self.nshift = 1

    def layout(self, side):
        return self.n, self.n

    def phases(self, ksc, side):
        return np.ones((np.atleast_2d(ksc).shape[0], 1, self.n), dtype=np.complex128)


def _run(b, E, p, electron):
    n = b["HL"].shape[-1]
    return transport_tdb_modes(E, b, RibbonLeads(n), np.zeros((1, 3)), lambda_eta=1e-3, a_z_l=1.0, a_z_r=1.0,
                               electron=electron, check=True, **p)


def test_electron_mode_sums_equal_caroli(cuda_ready):
    b, E, p = S.tb_ribbon(W=12, L=20, ne=64, disorder=0.5, eta=1e-9)
    E = E[(np.abs(E) > 0.05)]      # keep away from E = 0 exactly
    r = _run(b, E, p, electron=True)
    tot_l = r["transl_s"] + r["transl_ns"]
    tot_r = r["transr_s"] + r["transr_ns"]
    np.testing.assert_allclose(tot_l, r["transl"], rtol=1e-6, atol=1e-8)
    np.testing.assert_allclose(tot_r, r["transr"], rtol=1e-6, atol=1e-8)
    # unitarity: transmission + reflection of the left-incoming modes is their
    # (integer) number; evanescent modes within lambda_eta of the unit circle
    # near a subband edge may be counted as propagating, so the count bounds it
    refl = r["refll_s"] + r["refll_ns"]
    tr = r["transr"] + refl
    assert np.abs(tr - np.round(tr)).max() < 1e-5
    assert np.all(np.round(tr) <= r["nprop"][:, 0])
    assert (E < 0).any() and (E > 0).any()


def test_pristine_ribbon_counts_channels(cuda_ready):
    b, E, p = S.tb_ribbon(W=8, L=10, ne=40, disorder=0.0, eta=1e-9)
    E = E[(np.abs(E) > 0.05)]
    r = _run(b, E, p, electron=True)
    T = r["transl_s"] + r["transl_ns"]
    assert np.abs(T - np.round(T)).max() < 1e-5
    assert np.all(np.round(T) <= r["nprop"][:, 0])
    assert np.mean(np.round(T) == r["nprop"][:, 0]) > 0.9


def test_electron_and_phonon_normalisations_agree_for_positive_energy(cuda_ready):
    b, E, p = S.tb_ribbon(W=10, L=16, ne=48, disorder=0.4, eta=1e-9)
    E = E[E > 0.05]
    re = _run(b, E, p, electron=True)
    rp = _run(b, E, p, electron=False)
    for k in SUM_NAMES:
        np.testing.assert_allclose(re[k], rp[k], rtol=1e-8, atol=1e-10)
