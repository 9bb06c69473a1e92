"""GPU mode-resolved transmission (pf_transport_tdb_modes_dev) against the
reference's golden si-si sums and the FP64 oracle of vel_mat_tdb."""
import numpy as np
import pytest

from phinfortran_gb300.modes import SUM_NAMES, LeadGeometry, transport_tdb_modes
from tests.sisi_case import sisi_blocks, sisi_params
from tests.test_modes_host import oracle_point_sums

pytestmark = pytest.mark.gpu

DEGENERATE = {(13, 24), (14, 24), (54, 24)}   # Gamma-point points with a basis-dependent split


def run_gpu(f, ks, E_idx=None):
    nb = tuple(int(x) for x in f["n_bloch"])
    b, p = int(f["buffer"]), int(f["period"])
    geo = LeadGeometry.from_qe(f["pos_all"], f["cell"], f["cell_all"], nb, b, p, b, p)
    bl = [sisi_blocks(f, k) for k in ks]
    stacked = {name: np.stack([x[name] for x in bl]) for name in bl[0]}
    E1 = f["E"] if E_idx is None else f["E"][E_idx]
    ie = np.arange(f["E"].size) if E_idx is None else np.asarray(E_idx)
    E = np.tile(E1, len(ks))
    q = np.repeat(np.arange(len(ks)), E1.size).astype(np.int32)
    zf = np.tile((ie == 0).astype(np.int32), len(ks))
    cell = f["cell"]
    r = transport_tdb_modes(E, stacked, geo, f["kgrid"][ks], qidx=q, zero_flag=zf, lambda_eta=5e-3,
                            a_z_l=cell[2, 2], a_z_r=cell[2, 2], **sisi_params(f))
    return r, ie


def test_modes_against_reference_output(cuda_ready, sisi):
    """All 61 omega at nine k points: every sum within 1e-6 of the
    reference's output (outside the degenerate Gamma points), the total
    within 1e-6 everywhere, and s + ns equal to the Caroli T."""
    f = sisi
    ks = [0, 3, 10, 17, 24, 30, 37, 44, 48]
    r, ie = run_gpu(f, ks)
    ne = ie.size
    for a, ik in enumerate(ks):
        sl = slice(a * ne, (a + 1) * ne)
        for k in SUM_NAMES:
            got = r[k][sl]
            ref = f[k][:, ik]
            bad = [i for i in range(ne) if abs(got[i] - ref[i]) > 1e-6 and (i, ik) not in DEGENERATE]
            assert not bad, (k, ik, bad[:5], got[bad[:5]], ref[bad[:5]])
        tot = r["transl_s"][sl] + r["transl_ns"][sl]
        gtot = f["transl_s"][:, ik] + f["transl_ns"][:, ik]
        assert np.abs(tot - gtot).max() < 1e-6
        assert np.abs(tot - r["transl"][sl]).max() < 1e-8 * max(1.0, r["transl"][sl].max())
        totr = r["transr_s"][sl] + r["transr_ns"][sl]
        assert np.abs(totr - r["transr"][sl]).max() < 1e-8 * max(1.0, r["transr"][sl].max())


def test_modes_against_oracle(cuda_ready, sisi):
    f = sisi
    ies = [1, 6, 20, 33, 47]
    for ik in (10, 37):
        r, _ = run_gpu(f, [ik], ies)
        for a, (o, T) in enumerate(oracle_point_sums(f, ik, ies)):
            for k in SUM_NAMES:
                assert abs(r[k][a] - o[k]) < 1e-8 * max(1.0, abs(o[k])), (ik, ies[a], k, r[k][a], o[k])
            nprop_or = [len(o["modes"][m]["prop"]) for m in ("adv_l", "ret_l", "ret_r", "adv_r")]
            assert list(r["nprop"][a]) == nprop_or


def test_pristine_channel_counts(cuda_ready, sisi):
    """si-si is a pristine lead-device-lead stack: T is an integer number of
    channels (within the eta = 1e-8 broadening) and never exceeds the
    propagating-mode count of the left lead.  The count can exceed T near a
    band edge, where evanescent modes with | |lambda| - 1 | < lambda_eta
    (|lambda| = 0.997 here) pass the reference's propagating test while
    carrying no current."""
    f = sisi
    r, ie = run_gpu(f, [0, 17, 48])
    T = r["transl"]
    n_adv_l = r["nprop"][:, 0]
    assert np.abs(T - np.round(T)).max() < 1e-3
    assert np.all(np.round(T) <= n_adv_l)
    assert np.mean(np.round(T) == n_adv_l) > 0.95
