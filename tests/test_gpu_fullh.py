"""Binary force-constant (full-Hamiltonian) path on the GPU against the
oracle (oracle/binfc.py): the dense D(q) of pf_gen_dyn (reference-layout
host entry) and pf_gen_dyn_dev at the zone centre and at general transverse
k, the lead matrices (nz = 1, in-layer Hermitised, coupling not), the block
slices of pf_dense_to_tdb_dev, and the transmission of the whole chain
(D(q) built, sliced and solved on the device) against the oracle's
full-Hamiltonian transmission."""
import numpy as np
import pytest

from oracle import binfc as O
from oracle import negf as N
from phinfortran_gb300 import fullh, systems as S
from phinfortran_gb300.transport import BLOCK_NAMES

pytestmark = pytest.mark.gpu

KPTS = np.array([[0.0, 0.0, 0.0], [0.25, 0.0, 0.0], [0.1, -0.35, 0.0], [0.5, 0.5, 0.0]])


@pytest.fixture(scope="module")
def case(cuda_ready):
    d = S.sc_bar_binary_fc(nx=2, ny=2, L=5)
    t = fullh.fc_tables(d["pos_sc"], d["pos"], d["cell"], 1, 1, d["n_uc"], d["nz"], d["nfc"], d["r_cutoff"])
    fc = O.asr_cutoff(d["fc"], d["pos_sc"], d["r_cutoff"], 1, 1, 1)
    Hs = [O.gen_dyn(k, fc, d["masses"], d["recivec"], t.num, t.idx, t.dr, 1, 1, d["n_uc"], d["nz"]) for k in KPTS]
    d.update(tables=t, fc_asr=fc, H_oracle=np.array(Hs))
    return d


def test_gen_dyn_host_entry_matches_oracle(case):
    H = fullh.gen_dyn_host(case["fc_asr"], case["tables"], case["masses"], case["recivec"], KPTS, 1, 1,
                           case["n_uc"], case["nz"])
    ref = case["H_oracle"]
    scale = np.abs(ref).max()
    assert np.abs(H - ref).max() < 1e-13 * scale
    assert np.abs(H - np.swapaxes(H.conj(), -1, -2)).max() == 0.0


def test_gen_dyn_device_entry_matches_host_entry(case):
    import torch
    F = fullh.FullH(case["fc_asr"], case["tables"], case["masses"], case["recivec"], 1, 1, case["n_uc"],
                    case["nz"], nl=case["nl"], nr=case["nr"], n_buffer_l=case["n_buffer_l"],
                    n_buffer_r=case["n_buffer_r"], layer_list=[case["nl"]] * 5)
    Hd = F.dynamical(KPTS).transpose(-1, -2).cpu().numpy()
    torch.cuda.synchronize()
    Hh = fullh.gen_dyn_host(case["fc_asr"], case["tables"], case["masses"], case["recivec"], KPTS, 1, 1,
                            case["n_uc"], case["nz"])
    assert np.array_equal(Hd, Hh)


def test_lead_matrices_match_oracle(cuda_ready):
    lead = S.sc_lead_binary_fc(nx=2, ny=2)
    t, tv = fullh.fc_tables(lead["pos_sc"], lead["pos"], lead["cell"], 1, 1, lead["n_uc"], 1, lead["nfc"],
                            lead["r_cutoff"], lead=True)
    args = (lead["masses"], lead["recivec"], KPTS, 1, 1, lead["n_uc"], 1)
    Hl = fullh.gen_dyn_host(lead["fc"], t, *args, hermitize=True)
    Hlv = fullh.gen_dyn_host(lead["fc"], tv, *args, hermitize=False)
    for q, k in enumerate(KPTS):
        rl, rlv = O.gen_dyn_lead(k, lead["fc"], lead["masses"], lead["recivec"], t.num, t.idx, t.dr, tv.num,
                                 tv.idx, tv.dr, 1, 1, lead["n_uc"])
        s = np.abs(rl).max()
        assert np.abs(Hl[q] - rl).max() < 1e-13 * s
        assert np.abs(Hlv[q] - rlv).max() < 1e-13 * s


def test_slices_and_transmission(case):
    import torch
    H0 = case["H_oracle"][0]
    ll = fullh.blockwise_setup(H0, case["nl"], case["nr"], case["n_buffer_l"], case["n_buffer_r"])
    F = fullh.FullH(case["fc_asr"], case["tables"], case["masses"], case["recivec"], 1, 1, case["n_uc"],
                    case["nz"], nl=case["nl"], nr=case["nr"], n_buffer_l=case["n_buffer_l"],
                    n_buffer_r=case["n_buffer_r"], layer_list=ll)
    H = F.dynamical(KPTS)
    dev, dims = F.blocks(H)
    n, nl, nr, L, nq = dims
    for q in range(nq):
        ref = O.dense_to_tdb(case["H_oracle"][q], ll, nl, nr, case["n_buffer_l"], case["n_buffer_r"], n=n)
        Hq = H[q].transpose(0, 1).cpu().numpy()
        mine = O.dense_to_tdb(Hq, ll, nl, nr, case["n_buffer_l"], case["n_buffer_r"], n=n)
        for k in BLOCK_NAMES:
            got = dev[k][q].cpu().numpy()
            got = got[..., 0] + 1j * got[..., 1]
            got = np.swapaxes(got, -1, -2)
            assert np.array_equal(got, mine[k]), k           # exact copy of the device matrix
            assert np.abs(got - ref[k]).max() <= 1e-13 * np.abs(ref["HL"]).max(), k
    torch.cuda.synchronize()
    wmax = 2 * np.sqrt(1.0 / 28.0 * S.FC_TO_THZ2)
    Es = (np.linspace(0.03, 0.97, 12) * wmax) ** 2
    E = np.tile(Es, nq)
    qidx = np.repeat(np.arange(nq, dtype=np.int32), Es.size)
    p = dict(eta=1e-6, eta0=0.0, convergence=1e-12, dev_factor=10.0)
    got = F.transport(E, KPTS, qidx, want_transr=True, **p)
    assert not got["status"].any()
    for q in range(nq):
        B = O.dense_to_tdb(case["H_oracle"][q], ll, nl, nr, case["n_buffer_l"], case["n_buffer_r"])
        o = N.transport(Es, B, **p)
        ref = o["transl"]
        assert np.allclose(got["transl"][q * Es.size:(q + 1) * Es.size], ref, rtol=1e-9, atol=1e-12), q
        # T_R from the right-to-left sweep of G_block (device.f90:289-560)
        assert np.allclose(got["transr"][q * Es.size:(q + 1) * Es.size], o["transr"], rtol=1e-9, atol=1e-12), q
    # at the zone centre the chain is the bar of the tdb workloads
    bar_T = N.transport(Es, case["bar_blocks"], **p)["transl"]
    assert np.allclose(got["transl"][:Es.size], bar_T, rtol=1e-9, atol=1e-12)


def test_host_entry_rejects_bad_tables(case):
    from phinfortran_gb300 import _abi
    t = case["tables"]
    bad = fullh.FcTables(t.num.copy(), t.idx.copy(), t.dr)
    bad.num[0, 0] += 1                     # num_mat no longer sums to the entry count
    with pytest.raises(_abi.PFError):
        fullh.gen_dyn_host(case["fc_asr"], bad, case["masses"], case["recivec"], KPTS[:1], 1, 1, case["n_uc"],
                           case["nz"])
