"""Binary force-constant (full-Hamiltonian) path on the host.

The oracle (oracle/binfc.py, restating negf/fc.f90:25-44, negf/dyn.f90:39-312,
917-1271 and negf/device.f90:11-249) has no golden output in the reference
(its only example uses the QE force constants), so it is checked against an
independently assembled model: the simple-cubic bar of the tdb workloads
(per-atom masses, per-bond springs) written as a binary sandwich force
constant.  Its dense D(q) sliced at blockwise_setup's layers must give the
bar's lead blocks and the bar's transmission; the lead tables and
gen_dyn_lead must give the bar's lead cell and coupling.  The package's
host set-up (index tables through a k-d tree, the layer partition) must
equal the oracle's loops exactly.
"""
import numpy as np
import pytest

from oracle import binfc as O
from oracle import negf as N
from phinfortran_gb300 import fullh, systems as S


@pytest.fixture(scope="module")
def bar():
    d = S.sc_bar_binary_fc(nx=2, ny=2, L=4)
    num, idx, dr = O.fc_to_dyn_idx(d["pos_sc"], d["pos"], d["cell"], 1, 1, d["n_uc"], d["nz"], d["nfc"],
                                   d["r_cutoff"])
    fc = O.asr_cutoff(d["fc"], d["pos_sc"], d["r_cutoff"], 1, 1, 1)
    d.update(num=num, idx=idx, dr=dr, fc_asr=fc)
    return d


def test_read_binary_fc_column_major(tmp_path):
    a = np.random.default_rng(1).standard_normal((6, 15))
    p = tmp_path / "fc.bin"
    a.T.astype("<f8").tofile(p)          # Fortran stream write of a(6, 15): column-major
    assert np.array_equal(O.read_binary_fc(str(p), 6, 15), a)
    with pytest.raises(ValueError):
        O.read_binary_fc(str(p), 6, 16)


def test_fc_sc_positions_order():
    pos = np.array([[0.0, 0.0, 0.0, 1], [0.5, 0.5, 0.5, 2]])
    cell = np.diag([1.0, 2.0, 3.0])
    sc = O.fc_sc_positions(pos, 1, 1, 1, cell)
    assert sc.shape == (54, 4)
    # cell (i, j, k) = (1, -1, 0): ((1+1)*9 + (-1+1)*3 + 1 + 0) * 2
    base = (2 * 9 + 0 + 1) * 2
    assert np.allclose(sc[base + 1, :3], [1.5, -1.5, 0.5]) and sc[base + 1, 3] == 2


def test_asr_cutoff_zeroes_and_sums(bar):
    fc = bar["fc"].copy()
    fc[0, 3 * 100] = 0.3                       # a far pair: zeroed by the cutoff
    out = O.asr_cutoff(fc, bar["pos_sc"], bar["r_cutoff"], 1, 1, 1)
    assert out[0, 300] == 0.0
    rows = out.reshape(out.shape[0], -1, 3)
    assert np.abs(rows.sum(axis=1)).max() < 1e-12   # acoustic sum rule per (row, column component)
    assert np.abs(bar["fc_asr"] - bar["fc"]).max() < 1e-14


def test_tables_package_equals_oracle(bar):
    t = fullh.fc_tables(bar["pos_sc"], bar["pos"], bar["cell"], 1, 1, bar["n_uc"], bar["nz"], bar["nfc"],
                        bar["r_cutoff"])
    assert np.array_equal(t.num, bar["num"]) and np.array_equal(t.idx, bar["idx"])
    assert np.array_equal(t.dr, bar["dr"])
    a, b, off = t.pairs()
    assert off[-1] == t.idx.size and np.all(t.num[a, b] == np.diff(off))


def test_lead_tables_and_gen_dyn_lead(bar):
    lead = S.sc_lead_binary_fc(nx=2, ny=2)
    num, idx, dr, nv, iv, dv = O.lead_fc_to_dyn_idx(lead["pos_sc"], lead["pos"], lead["cell"], 1, 1,
                                                    lead["n_uc"], lead["nfc"], lead["r_cutoff"])
    t, tv = fullh.fc_tables(lead["pos_sc"], lead["pos"], lead["cell"], 1, 1, lead["n_uc"], 1, lead["nfc"],
                            lead["r_cutoff"], lead=True)
    assert np.array_equal(t.num, num) and np.array_equal(t.idx, idx) and np.array_equal(t.dr, dr)
    assert np.array_equal(tv.num, nv) and np.array_equal(tv.idx, iv) and np.array_equal(tv.dr, dv)
    Hl, Hlv = O.gen_dyn_lead([0, 0, 0], lead["fc"], lead["masses"], lead["recivec"], num, idx, dr, nv, iv, dv,
                             1, 1, lead["n_uc"])
    bb = bar["bar_blocks"]
    scale = np.abs(bb["HL"]).max()
    assert np.abs(Hl - bb["HL"]).max() < 1e-14 * scale
    assert np.abs(Hlv - bb["HLv"]).max() < 1e-14 * scale
    H = O.gen_dyn([0, 0, 0], bar["fc_asr"], bar["masses"], bar["recivec"], bar["num"], bar["idx"], bar["dr"],
                  1, 1, bar["n_uc"], bar["nz"])
    Hs = O.swap_lead_region(H, Hl, Hl, Hlv, Hlv, bar["n_uc"], 4, 4, 4, 4)
    assert np.abs(Hs - H).max() < 1e-13 * scale     # the sandwich already holds bulk lead cells


def test_gen_dyn_hermitian_and_bloch_phase(bar):
    args = (bar["fc_asr"], bar["masses"], bar["recivec"], bar["num"], bar["idx"], bar["dr"], 1, 1,
            bar["n_uc"], bar["nz"])
    H0 = O.gen_dyn([0, 0, 0], *args)
    Hk = O.gen_dyn([0.25, 0.1, 0.0], *args)
    assert np.abs(Hk - Hk.conj().T).max() == 0.0
    assert np.abs(Hk - H0).max() > 1e-3 * np.abs(H0).max()   # the transverse phase acts
    # acoustic sum rule at k = 0: sum_b sqrt(m_b) D(a i, b j) = 0
    m3 = np.repeat(bar["masses"], 3)
    assert np.abs((H0 * np.sqrt(m3)[None, :]).reshape(-1, bar["n_uc"], 3).sum(axis=1)).max() < 1e-10


def test_blockwise_setup_package_equals_oracle(bar):
    H = O.gen_dyn([0, 0, 0], bar["fc_asr"], bar["masses"], bar["recivec"], bar["num"], bar["idx"], bar["dr"],
                  1, 1, bar["n_uc"], bar["nz"])
    args = (bar["nl"], bar["nr"], bar["n_buffer_l"], bar["n_buffer_r"])
    ll = O.blockwise_setup(H, *args)
    assert ll == fullh.blockwise_setup(H, *args)
    assert sum(ll) == H.shape[0] - 2 * bar["n_buffer_l"] - 4 * bar["nl"]
    rng = np.random.default_rng(3)
    for trial in range(6):
        # random banded Hermitian matrices with a varying band: exercises both branches of the scan
        nb, nl = 4, 5
        nd = 40
        norb = 2 * nb + 4 * nl + nd
        A = np.zeros((norb, norb), np.complex128)
        w = rng.integers(2, 9, size=norb)
        for i in range(norb):
            for j in range(i, min(norb, i + w[i])):
                A[i, j] = rng.standard_normal() + 1j * rng.standard_normal()
        A = A + A.conj().T
        assert O.blockwise_setup(A, nl, nl, nb, nb) == fullh.blockwise_setup(A, nl, nl, nb, nb), trial


def test_full_h_transmission_equals_bar(bar):
    H = O.gen_dyn([0, 0, 0], bar["fc_asr"], bar["masses"], bar["recivec"], bar["num"], bar["idx"], bar["dr"],
                  1, 1, bar["n_uc"], bar["nz"])
    ll = O.blockwise_setup(H, bar["nl"], bar["nr"], bar["n_buffer_l"], bar["n_buffer_r"])
    B = O.dense_to_tdb(H, ll, bar["nl"], bar["nr"], bar["n_buffer_l"], bar["n_buffer_r"])
    bb = bar["bar_blocks"]
    for k in ("HL", "HLv", "HR", "HRv"):
        assert np.abs(B[k] - bb[k]).max() < 1e-14 * np.abs(bb["HL"]).max(), k
    wmax = 2 * np.sqrt(1.0 / 28.0 * S.FC_TO_THZ2)
    E = (np.linspace(0.05, 0.95, 9) * wmax) ** 2
    p = dict(eta=1e-6, eta0=0.0, convergence=1e-12, dev_factor=10.0)
    t1 = N.transport(E, B, **p)["transl"]
    t2 = N.transport(E, bb, **p)["transl"]
    assert np.allclose(t1, t2, rtol=1e-9, atol=1e-12)
    assert t1[0] > 3.9   # four acoustic-branch channels open near the band bottom


def test_row_atoms_matches_reference_decomposition():
    nbx, nby, n_uc, nz = 2, 3, 12, 4
    natoms = nbx * nby * n_uc
    per = n_uc // nz
    ref = []
    for a in range(natoms):       # negf/dyn.f90:95-103 with 1-based atm_idx_s = a + 1
        a1 = a + 1
        iz = (a1 - 1) // (nby * nbx * per)
        iy = (a1 - iz * (nby * nbx * per) - 1) // (nbx * per)
        ix = (a1 - iz * (nby * nbx * per) - iy * (nbx * per) - 1) // per
        is1 = a1 - iz * (nby * nbx * per) - iy * (nbx * per) - ix * per
        ref.append(iz * per + is1 - 1)
    assert np.array_equal(fullh.row_atoms(natoms, nbx, nby, n_uc, nz), ref)
