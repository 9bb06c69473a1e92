"""Mode-to-mode matrices (pf_transport_tdb_modes_md2md_dev) and the files of
write_md2md (negf/write_data.f90:177-241, verbosity = 1) on the si-si case.

The reference ships no md2md files, and the split of |M_ij|^2 among
degenerate modes depends on the eigen-solver's basis, so the matrices are
checked through what is basis-independent and already pinned: their
label-matched and label-crossing sums are the eight s/ns sums of the same
run, their label-grouped column sums are col_sums, and the rows of the
written files add up to the row and column totals."""
import numpy as np
import pytest

from phinfortran_gb300.modes import KINDS, MATRICES, MD2MD_FILES, LeadGeometry, md2md_rows, transport_tdb_modes
from phinfortran_gb300.output import write_md2md_files
from tests.sisi_case import sisi_blocks, sisi_params, sisi_primitive_cell

pytestmark = pytest.mark.gpu

# matrix -> (row problem, column problem, s sum, ns sum)
SPLIT = {"tlr": ("ret_l", "adv_r", "transl_s", "transl_ns"), "trl": ("ret_r", "adv_l", "transr_s", "transr_ns"),
         "rrr": ("ret_r", "adv_r", "reflr_s", "reflr_ns"), "rll": ("ret_l", "adv_l", "refll_s", "refll_ns")}


def test_md2md_matrices_and_files(cuda_ready, sisi, tmp_path):
    f = sisi
    ks = [4, 30]
    nb = tuple(int(x) for x in f["n_bloch"])
    b, p = int(f["buffer"]), int(f["period"])
    geo = LeadGeometry.from_qe(f["pos_all"], f["cell"], f["cell_all"], nb, b, p, b, p)
    bl = [sisi_blocks(f, k) for k in ks]
    stacked = {name: np.stack([x[name] for x in bl]) for name in bl[0]}
    E1 = f["E"][5:60:6]
    E = np.tile(E1, len(ks))
    q = np.repeat(np.arange(len(ks)), E1.size).astype(np.int32)
    cell = f["cell"]
    r = transport_tdb_modes(E, stacked, geo, f["kgrid"][ks], qidx=q, lambda_eta=5e-3, a_z_l=cell[2, 2],
                            a_z_r=cell[2, 2], md2md=True, **sisi_params(f))
    M = r["md2md"]
    assert M.shape == (E.size, 4, r["nl"], r["nl"])
    bz = r["mode_bz"]
    for mat, (rk, ck, s_key, ns_key) in SPLIT.items():
        m = MATRICES.index(mat)
        br, bc = bz[:, KINDS.index(rk)], bz[:, KINDS.index(ck)]
        both = (br[:, :, None] > 0) & (bc[:, None, :] > 0)
        same = both & (br[:, :, None] == bc[:, None, :])
        s = (M[:, m] * same).sum(axis=(1, 2))
        ns = (M[:, m] * (both & ~same)).sum(axis=(1, 2))
        tol = 1e-12 + 1e-10 * np.abs(r[s_key]).max()
        assert np.abs(s - r[s_key]).max() <= tol, mat
        assert np.abs(ns - r[ns_key]).max() <= 1e-12 + 1e-10 * max(np.abs(r[ns_key]).max(), 1.0), mat
        # label-grouped column sums of the same matrix
        for lab in range(1, geo.nshift + 1):
            cs = (M[:, m] * ((br[:, :, None] == lab) & (bc[:, None, :] > 0))).sum(axis=1)
            assert np.abs(cs - r["col_sums"][:, m, :, lab - 1]).max() <= 1e-12, (mat, lab)
    assert r["transl_s"].max() > 1.0
    rows = md2md_rows(r, geo, f["kgrid"][ks], E, qidx=q, pc=sisi_primitive_cell(f))
    write_md2md_files(str(tmp_path), rows, k_index={a: k + 1 for a, k in enumerate(ks)})
    for d, (mat, rk, ck) in MD2MD_FILES.items():
        m = MATRICES.index(mat)
        kz = r["mode_kz"]
        n_rows = sum(len(rr) for qq, rr in rows[d] if qq == 0)
        prop = [(int(((kz[i, KINDS.index(rk)] < 99.9) & (bz[i, KINDS.index(rk)] > 0)).sum()),
                 int(((kz[i, KINDS.index(ck)] < 99.9) & (bz[i, KINDS.index(ck)] > 0)).sum()))
                for i in range(E.size) if q[i] == 0]
        assert n_rows == sum(a * c for a, c in prop)
        a = np.loadtxt(tmp_path / f"{d}_md2md_{ks[0] + 1:06d}.dat", ndmin=2)
        assert a.shape == (n_rows, 25)
        # ts + tns of every pair is |M_ij|^2; per point they add up to the
        # whole propagating block of the matrix
        start = 0
        for i in np.nonzero(q == 0)[0]:
            cnt = prop[list(np.nonzero(q == 0)[0]).index(i)]
            blk = a[start:start + cnt[0] * cnt[1]]
            start += cnt[0] * cnt[1]
            pr = (kz[i, KINDS.index(rk)] < 99.9) & (bz[i, KINDS.index(rk)] > 0)
            pc_ = (kz[i, KINDS.index(ck)] < 99.9) & (bz[i, KINDS.index(ck)] > 0)
            want = M[i, m][np.ix_(pr, pc_)].sum()
            assert abs(blk[:, 21].sum() + blk[:, 22].sum() - want) <= 1e-9 * max(want, 1.0), d
            if len(blk):
                assert (blk[:, 2] == blk[0, 2]).all() and abs(blk[0, 2] - np.sqrt(E[i])) < 1e-8
