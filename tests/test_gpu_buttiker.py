"""Buttiker probes on the GPU (pf_buttiker_tdb) against the oracle
(oracle/buttiker.py): per point T_L, probe and lead fluxes, Tr A_i, Tr Gn_i
and the full Jacobian, including the zero-frequency point and two q block
sets in one call; and the Newton iteration on the probe temperatures
against the oracle's loop."""
import numpy as np
import pytest

from oracle import buttiker as BP
from phinfortran_gb300 import buttiker as PB
from phinfortran_gb300 import systems as S

pytestmark = pytest.mark.gpu

B_PROBE = 5.0e-20 * (2.0 * 3.1415926 * 1.0e12) * 1.0e3


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module")
def bars(cuda_ready):
    b1, E, p, _ = S.sc_phonon(nx=2, ny=2, L=5, ne=33, mass_range=(1.0, 2.0), seed_index=1)
    b2, _, _, _ = S.sc_phonon(nx=2, ny=2, L=5, ne=33, mass_range=(1.0, 2.0), seed_index=7)
    Eg = np.concatenate([[1.0e-6], E[:32]])          # 33 energies, the first one the zero-frequency point
    return b1, b2, Eg, p


def test_points_match_oracle(bars):
    b1, b2, Eg, p = bars
    L = b1["Hd"].shape[0]
    temps = BP.initial_temperatures(L, 300.0, 310.0) + np.array([0.3, -0.2, 0.1, 0.0, 0.4])
    sw, dsw = BP.set_sigma_bp_w(temps, Eg, B_PROBE, 430.0)
    first = np.arange(Eg.size) == 0
    stack = {k: np.stack([b1[k], b2[k]]) for k in b1}
    E = np.tile(Eg, 2)
    q = np.repeat(np.arange(2, dtype=np.int32), Eg.size)
    got = PB.probe_points(E, stack, np.tile(sw.T, (2, 1)), np.tile(dsw.T, (2, 1)), temps, 300.0, 310.0,
                          qidx=q, first=np.tile(first, 2).astype(np.int32), eta=p["eta"], eta0=p["eta0"],
                          convergence=p["convergence"])
    for k, b in enumerate((b1, b2)):
        ref = BP.probe_point_batch(Eg, first, b, sw.T, dsw.T, temps, 300.0, 310.0, p["eta"], p["eta0"],
                                   p["convergence"])
        s = slice(k * Eg.size, (k + 1) * Eg.size)
        assert np.allclose(got["transl"][s], ref["transl"], rtol=1e-9, atol=1e-12)
        for key in ("flux_i", "A_sum", "Gn_i", "flux_left", "flux_right"):
            assert rel(got[key][s], ref[key]) < 1e-9, key
        assert rel(got["jacobian"][s], ref["jacobian"]) < 1e-9
        assert not got["jacobian"][s][0].any() and not got["flux_i"][s][0].any()


def test_newton_loop_matches_oracle(bars):
    b1, _, Eg, p = bars
    kw = dict(eta=p["eta"], eta0=p["eta0"], convergence=p["convergence"])
    mine = PB.probe_loop(Eg, [b1], 300.0, 310.0, B_PROBE, 430.0, max_iter=4, **kw)
    ref = BP.probe_loop(Eg, [b1], 300.0, 310.0, B_PROBE, 430.0, max_iter=4, **kw)
    assert mine["iterations"] == ref["iterations"]
    assert np.allclose(mine["temps"], ref["temps"], rtol=0, atol=1e-7)
    assert np.allclose(mine["temps_ph"], ref["temps_ph"], rtol=0, atol=1e-6)
