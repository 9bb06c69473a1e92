"""Mode-resolved transmission through pf_transport_tdb_modes_dev.

The reference computes, per (omega^2, k) point, the Bloch eigenmodes of
the lead transfer matrices, the t/r matrices between them and the split of
transmission / reflection into specular (same folded-BZ label) and
non-specular parts (vel_mat_tdb, negf/velocity_mat.f90:1692-3148).  The
GPU entry does all of it; this module prepares the geometry the unfolding
needs and calls it:

* ``LeadGeometry.from_qe`` restates transverse_uc_setup
  (velocity_mat.f90:14-179) in its qe_fc form (positions = the supercell
  atoms, latvec_uc = the QE cell; negf/phinfortran.f90:122-160);
* ``LeadGeometry.phases`` gives, per k point, the unfolding phase of every
  lead orbital for every folded shift (velocity_mat.f90:2035-2072,
  move_in_ws2 of util.f90:675-706 for the shifted k).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from .transport import BLOCK_NAMES, TdbBlocks, fortran_block

SUM_NAMES = ("transl_s", "transl_ns", "transr_s", "transr_ns", "refll_s", "refll_ns", "reflr_s", "reflr_ns")


def _move_in_ws2(k, a):
    """The in-plane translate k - (i1 a1 + i2 a2), |i| <= 2, closest to 0;
    first minimum with i1 outer (util.f90:675-706)."""
    best, out = None, None
    for i1 in range(-2, 3):
        for i2 in range(-2, 3):
            d = k - (i1 * a[0] + i2 * a[1])
            dd = float(d @ d)
            if best is None or dd < best:
                best, out = dd, d
    return out


def _lead_side(pos_all, atoms, cell_uc, nb, tol):
    inv_uc = np.linalg.inv(cell_uc)
    reps = [i for i in atoms if -0.001 < (pos_all[i] @ inv_uc)[0] < 0.999
            and -0.001 < (pos_all[i] @ inv_uc)[1] < 0.999]
    pos, rep_of = [], []
    temp = 0
    for i in atoms:
        for j, a in enumerate(reps):
            for kx in range(nb[0]):
                for ky in range(nb[1]):
                    dp = pos_all[i] - pos_all[a] - (kx * cell_uc[0] + ky * cell_uc[1])
                    if np.sqrt(dp @ dp) < tol:
                        temp = j
        for _ in range(3):
            pos.append(pos_all[i])
            rep_of.append(temp)
    return np.array(pos), np.array(rep_of, dtype=np.int64), np.array(reps, dtype=np.int64)


@dataclass
class LeadGeometry:
    """Orbital positions and transverse-cell representatives of both leads."""
    pos_all: np.ndarray
    cell_uc: np.ndarray
    cell_all: np.ndarray
    n_bloch: tuple
    pos_l: np.ndarray
    rep_l: np.ndarray
    list_l: np.ndarray
    pos_r: np.ndarray
    rep_r: np.ndarray
    list_r: np.ndarray

    @classmethod
    def from_qe(cls, pos_all, cell_uc, cell_all, n_bloch, buffer_left, period_left, buffer_right, period_right):
        pos_all = np.asarray(pos_all, dtype=np.float64)
        nb = (int(n_bloch[0]), int(n_bloch[1]))
        na = pos_all.shape[0]
        pl, rl, ll = _lead_side(pos_all, range(buffer_left + period_left, buffer_left + 2 * period_left),
                                cell_uc, nb, 1.0e-3)
        pr, rr, lr = _lead_side(pos_all, range(na - buffer_right - 2 * period_right, na - buffer_right - period_right),
                                cell_uc, nb, 1.0e-5)
        return cls(pos_all, np.asarray(cell_uc, float), np.asarray(cell_all, float), nb, pl, rl, ll, pr, rr, lr)

    @property
    def nshift(self):
        return self.n_bloch[0] * self.n_bloch[1]

    def layout(self, side):
        """(stride, nrep): orbital stride between transverse images and the
        orbitals of the first image that the unfolding sums over."""
        pos = self.pos_l if side == "l" else self.pos_r
        lst = self.list_l if side == "l" else self.list_r
        n = pos.shape[0]
        return n // self.nshift, 3 * lst.size

    def phases(self, ksc, side):
        """(nk, nshift, n) complex phases exp(-i(-p.k_sc + (p - p_uc).k_j))."""
        ksc = np.atleast_2d(np.asarray(ksc, dtype=np.float64))
        recivec = 2 * np.pi * np.linalg.inv(self.cell_all).T
        reci_uc = 2 * np.pi * np.linalg.inv(self.cell_uc).T
        pos = self.pos_l if side == "l" else self.pos_r
        rep = self.rep_l if side == "l" else self.rep_r
        lst = self.list_l if side == "l" else self.list_r
        stride, nrep = self.layout(side)
        n = pos.shape[0]
        shifts = [(i, j) for i in range(self.n_bloch[0]) for j in range(self.n_bloch[1])]
        out = np.zeros((ksc.shape[0], len(shifts), n), dtype=np.complex128)
        rows = np.arange(n)
        r0 = rows % stride
        ok = r0 < nrep
        # representative atom of the first-image orbital each row belongs to
        pos_uc = self.pos_all[lst[rep[r0 - (r0 % 3)]]]
        for ik, k in enumerate(ksc):
            kc = k @ recivec
            for js, (sx, sy) in enumerate(shifts):
                kp = _move_in_ws2((np.array([sx, sy, 0.0]) + k) @ recivec, reci_uc)
                ph = np.exp(-1j * (-(pos @ kc) + np.einsum("ij,j->i", pos - pos_uc, kp)))
                out[ik, js] = np.where(ok, ph, 0.0)
        return out


def transport_tdb_modes(E, blocks, geometry, ksc, *, eta, eta0, convergence, lambda_eta, a_z_l, a_z_r,
                        dev_factor=10.0, qidx=None, zero_flag=None, max_iter=1000, check=True):
    """Transmission and its mode-resolved split for a batch of points.

    ``blocks``: one q (dict) or a TdbBlocks stack; ``ksc``: (nq, 3)
    fractional k of every q block (the reference's k_grid rows).  Returns a
    dict with transl, transr, the eight sums of SUM_NAMES, nprop (npts, 4)
    and status.
    """
    import torch
    lib = _abi.load()
    if isinstance(blocks, dict):
        blocks = TdbBlocks.from_dict(blocks)
    nq, (n, nl, nr, L), arrs = blocks.stacked()
    ksc = np.atleast_2d(np.asarray(ksc, dtype=np.float64))
    if ksc.shape[0] != nq:
        raise ValueError("one k point per q block")
    dev = {k: torch.from_numpy(fortran_block(v).copy()).cuda() for k, v in arrs.items()}
    E = np.ascontiguousarray(E, dtype=np.float64)
    npts = E.size
    ph_l = torch.from_numpy(np.ascontiguousarray(geometry.phases(ksc, "l")).view(np.float64).copy()).cuda()
    ph_r = torch.from_numpy(np.ascontiguousarray(geometry.phases(ksc, "r")).view(np.float64).copy()).cuda()
    sl, rl_ = geometry.layout("l")
    sr, rr_ = geometry.layout("r")
    Ed = torch.from_numpy(E).cuda()
    qd = None if qidx is None else torch.from_numpy(np.ascontiguousarray(qidx, dtype=np.int32)).cuda()
    zd = None if zero_flag is None else torch.from_numpy(np.ascontiguousarray(zero_flag, dtype=np.int32)).cuda()
    tl = torch.zeros(max(npts, 1), dtype=torch.float64, device="cuda")
    tr = torch.zeros_like(tl)
    sums = torch.zeros((max(npts, 1), 8), dtype=torch.float64, device="cuda")
    st = torch.zeros(max(npts, 1), dtype=torch.int32, device="cuda")
    npr = torch.zeros((max(npts, 1), 4), dtype=torch.int32, device="cuda")
    ws = lib.pf_transport_tdb_modes_workspace_size(n, nl, nr, nq, npts)
    if ws == 0:
        raise _abi.PFError(-3, "mode-resolved kernel does not fit (block size > 48?)")
    work = torch.empty(ws, dtype=torch.uint8, device="cuda")
    p = lambda t: None if t is None else t.data_ptr()
    rc = lib.pf_transport_tdb_modes_dev(n, nl, nr, L, nq, *[dev[k].data_ptr() for k in BLOCK_NAMES], npts,
                                        Ed.data_ptr(), p(qd), p(zd), eta, eta0, dev_factor, convergence, max_iter,
                                        lambda_eta, a_z_l, a_z_r, geometry.nshift, sl, rl_, ph_l.data_ptr(), sr, rr_,
                                        ph_r.data_ptr(), tl.data_ptr(), tr.data_ptr(), sums.data_ptr(), st.data_ptr(),
                                        npr.data_ptr(), work.data_ptr(), ws,
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc != 0:
        raise _abi.PFError(rc, lib.pf_modes_last_error().decode(errors="replace"))
    torch.cuda.synchronize()
    status = st.cpu().numpy()[:npts]
    if check and (status != 0).any():
        raise _abi.PFError(-4, f"point status flags 0x{int(np.bitwise_or.reduce(status)):x}")
    s = sums.cpu().numpy()[:npts]
    out = dict(transl=tl.cpu().numpy()[:npts], transr=tr.cpu().numpy()[:npts], nprop=npr.cpu().numpy()[:npts],
               status=status)
    for i, k in enumerate(SUM_NAMES):
        out[k] = s[:, i].copy()
    return out
