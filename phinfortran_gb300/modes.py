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
  move_in_ws2 of util.f90:675-706 for the shifted k);
* ``mode_rows`` turns the per-mode outputs (``per_mode=True``) into the
  rows of the reference's per-k mode files (write_specular / write_md,
  negf/write_data.f90:3-176, called at velocity_mat.f90:3108-3128), which
  ``output.write_mode_files`` writes.
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

    def label_k(self, ksc):
        """(nshift, 3) Cartesian in-plane k of every unfolding label for the
        fractional k ``ksc``: move_in_ws2((ksc + shift) . recivec, reci_uc)
        (velocity_mat.f90:2353-2356; z is replaced by the mode's k_z)."""
        recivec = 2 * np.pi * np.linalg.inv(self.cell_all).T
        reci_uc = 2 * np.pi * np.linalg.inv(self.cell_uc).T
        shifts = [(i, j) for i in range(self.n_bloch[0]) for j in range(self.n_bloch[1])]
        k = np.asarray(ksc, dtype=np.float64)
        return np.array([_move_in_ws2((np.array([sx, sy, 0.0]) + k) @ recivec, reci_uc) for sx, sy in shifts])

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
                        dev_factor=10.0, qidx=None, zero_flag=None, max_iter=1000, check=True, per_mode=False,
                        electron=False, md2md=False):
    """Transmission and its mode-resolved split for a batch of points.

    ``blocks``: one q (dict) or a TdbBlocks stack; ``ksc``: (nq, 3)
    fractional k of every q block (the reference's k_grid rows).  Returns a
    dict with transl, transr, the eight sums of SUM_NAMES, nprop (npts, 4)
    and status; with ``per_mode`` also mode_kz, mode_bz (npts, 4, mm) and
    col_sums (npts, 4, mm, nshift) of pf_transport_tdb_modes_permode_dev
    (problems adv-L, ret-L, ret-R, adv-R; matrices tlr, trl, rrr, rll).
    ``electron`` selects the tight-binding normalisation (velocity matrices
    and t / r without the phonon a_z / (2 sqrt(E)) factors; energies may be
    negative).  ``md2md`` (implies ``per_mode``) adds the whole mode-to-mode
    matrices |M_rc|^2 as md2md (npts, 4, mm rows, mm columns)
    (pf_transport_tdb_modes_md2md_dev), what write_md2md prints.
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
    head = (n, nl, nr, L, nq, *[dev[k].data_ptr() for k in BLOCK_NAMES], npts, Ed.data_ptr(), p(qd), p(zd), eta,
            eta0, dev_factor, convergence, max_iter, lambda_eta, a_z_l, a_z_r, geometry.nshift, sl, rl_,
            ph_l.data_ptr(), sr, rr_, ph_r.data_ptr())
    outs = (tl.data_ptr(), tr.data_ptr(), sums.data_ptr(), st.data_ptr(), npr.data_ptr())
    tail = (work.data_ptr(), ws, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    flags = 1 if electron else 0   # PF_MODES_ELECTRON
    per_mode = per_mode or md2md
    if per_mode:
        mm = max(nl, nr)
        kz = torch.zeros((max(npts, 1), 4, mm), dtype=torch.float64, device="cuda")
        bz = torch.zeros((max(npts, 1), 4, mm), dtype=torch.int32, device="cuda")
        cs = torch.zeros((max(npts, 1), 4, mm, geometry.nshift), dtype=torch.float64, device="cuda")
        m2 = torch.zeros((max(npts, 1), 4, mm, mm), dtype=torch.float64, device="cuda") if md2md else None
        rc = lib.pf_transport_tdb_modes_md2md_dev(*head, flags, *outs, kz.data_ptr(), bz.data_ptr(),
                                                  cs.data_ptr(), p(m2), *tail)
    else:
        rc = lib.pf_transport_tdb_modes_ex_dev(*head, flags, *outs, None, None, None, *tail)
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
    if per_mode:
        out.update(mode_kz=kz.cpu().numpy()[:npts], mode_bz=bz.cpu().numpy()[:npts],
                   col_sums=cs.cpu().numpy()[:npts], nl=nl, nr=nr)
        if md2md:
            # device layout [p][matrix][column][row] -> (npts, 4, rows, columns)
            out["md2md"] = np.ascontiguousarray(np.swapaxes(m2.cpu().numpy()[:npts], -1, -2))
    return out


BLOCK_OUTPUTS = ("gl_adv", "gl_plus", "gr_ret", "gr_minus", "gml_adv", "gmr_ret", "G_D_LR", "G_R", "G_D_RL", "G_L")


def transport_tdb_blocks(E, blocks, *, eta, eta0, convergence, dev_factor=10.0, qidx=None, zero_flag=None,
                         max_iter=1000, want=BLOCK_OUTPUTS, check=True):
    """FP64 transmission plus the Green's-function blocks that vel_mat_tdb
    receives (pf_transport_tdb_blocks_dev): the surface functions gl_adv,
    gl_plus, gr_ret, gr_minus, the broadenings gml_adv, gmr_ret, and
    G_D_LR = G_{0,N+1}, G_R, G_D_RL = G_{N+1,0}, G_L.  ``want`` names the
    blocks to return (complex (npts, rows, cols) arrays); the others are not
    written on the device.  Also returns transl, transr and status."""
    import torch
    lib = _abi.load()
    if isinstance(blocks, dict):
        blocks = TdbBlocks.from_dict(blocks)
    nq, (n, nl, nr, L), arrs = blocks.stacked()
    unknown = set(want) - set(BLOCK_OUTPUTS)
    if unknown:
        raise ValueError(f"unknown blocks {sorted(unknown)}")
    dev = {k: torch.from_numpy(fortran_block(v).copy()).cuda() for k, v in arrs.items()}
    E = np.ascontiguousarray(E, dtype=np.float64)
    npts = E.size
    Ed = torch.from_numpy(E).cuda()
    qd = None if qidx is None else torch.from_numpy(np.ascontiguousarray(qidx, dtype=np.int32)).cuda()
    zd = None if zero_flag is None else torch.from_numpy(np.ascontiguousarray(zero_flag, dtype=np.int32)).cuda()
    tl = torch.zeros(max(npts, 1), dtype=torch.float64, device="cuda")
    tr = torch.zeros_like(tl)
    st = torch.zeros(max(npts, 1), dtype=torch.int32, device="cuda")
    shapes = dict(gl_adv=(nl, nl), gl_plus=(nl, nl), gr_ret=(nr, nr), gr_minus=(nr, nr), gml_adv=(nl, nl),
                  gmr_ret=(nr, nr), G_D_LR=(nl, nr), G_R=(nr, nr), G_D_RL=(nr, nl), G_L=(nl, nl))
    bufs = {k: torch.zeros((max(npts, 1), shapes[k][1], shapes[k][0], 2), dtype=torch.float64, device="cuda")
            for k in want}
    ws = lib.pf_transport_tdb_blocks_workspace_size(n, nl, nr, nq, npts)
    if ws == 0:
        raise _abi.PFError(-3, "kernel does not fit (block size > 48?)")
    work = torch.empty(ws, dtype=torch.uint8, device="cuda")
    p = lambda t: None if t is None else t.data_ptr()
    rc = lib.pf_transport_tdb_blocks_dev(n, nl, nr, L, nq, *[dev[k].data_ptr() for k in BLOCK_NAMES], npts,
                                         Ed.data_ptr(), p(qd), p(zd), eta, eta0, dev_factor, convergence, max_iter,
                                         tl.data_ptr(), tr.data_ptr(), st.data_ptr(),
                                         *[p(bufs.get(k)) for k in BLOCK_OUTPUTS], work.data_ptr(), ws,
                                         C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc != 0:
        raise _abi.PFError(rc, lib.pf_modes_last_error().decode(errors="replace"))
    torch.cuda.synchronize()
    status = st.cpu().numpy()[:npts]
    if check and (status != 0).any():
        raise _abi.PFError(-4, f"point status flags 0x{int(np.bitwise_or.reduce(status)):x}")
    out = dict(transl=tl.cpu().numpy()[:npts], transr=tr.cpu().numpy()[:npts], status=status)
    for k, v in bufs.items():
        a = v.cpu().numpy()[:npts]                      # (npts, cols, rows, 2): column-major blocks
        out[k] = np.transpose(a[..., 0] + 1j * a[..., 1], (0, 2, 1))
    return out


KINDS = ("adv_l", "ret_l", "ret_r", "adv_r")
MATRICES = ("tlr", "trl", "rrr", "rll")
# write_specular calls (velocity_mat.f90:3108-3120): file -> (matrix, incoming problem)
SPECULAR_FILES = {"tlr": ("tlr", "adv_r"), "trl": ("trl", "adv_l"), "right": ("rrr", "adv_r"),
                  "left": ("rll", "adv_l")}
# write_md calls (velocity_mat.f90:3121-3126): file -> (t matrix, r matrix, incoming problem)
MD_FILES = {"mdl": ("trl", "rll", "adv_l"), "mdr": ("tlr", "rrr", "adv_r")}
MODE_FILES = ("left", "right", "tlr", "trl", "mdl", "mdr")


def _clamp(x):
    return 1.0e-60 if 0.0 < x < 1.0e-60 else x


def _pc_columns(res, labk, q_of, E, pcs, kinds):
    """Primitive-cell k and velocity (npts, modes, 6) of the propagating
    modes of each problem kind, one unfolding batch per kind (zero without
    a primitive cell)."""
    size = {"adv_l": res["nl"], "ret_l": res["nl"], "ret_r": res["nr"], "adv_r": res["nr"]}
    npts = E.size
    pcol = {}
    for kind in kinds:
        side = 0 if kind.endswith("_l") else 1
        ki = KINDS.index(kind)
        cols = np.zeros((npts, size[kind], 6))
        if pcs[side] is not None:
            kz, bz = res["mode_kz"][:, ki, :size[kind]], res["mode_bz"][:, ki, :size[kind]]
            pp, ii = np.nonzero((kz < 99.9) & (bz > 0))
            if pp.size:
                lk = np.array([labk[int(q_of[a])][bz[a, i] - 1] for a, i in zip(pp, ii)])
                lk[:, 2] = kz[pp, ii]
                kp, vp = pcs[side].unfold(E[pp], lk)
                cols[pp, ii, :3], cols[pp, ii, 3:] = kp, vp
        pcol[kind] = cols
    return pcol


def _mode_k(res, p, kind, lk):
    """(modes, 3) k of every mode of one problem: the label's in-plane k
    with the mode's k_z, 100 for the modes that do not propagate."""
    size = res["nl"] if kind.endswith("_l") else res["nr"]
    ki = KINDS.index(kind)
    kz, bz = res["mode_kz"][p, ki], res["mode_bz"][p, ki]
    k = np.full((size, 3), 100.0)
    for i in range(size):
        if kz[i] < 99.9 and bz[i] > 0:
            k[i] = lk[bz[i] - 1]
            k[i, 2] = kz[i]
    return k


# write_md2md calls (velocity_mat.f90:3132-3145): file -> (matrix, row problem k_f, column problem k_b)
MD2MD_FILES = {"tlr": ("tlr", "ret_l", "adv_r"), "trl": ("trl", "ret_r", "adv_l"),
               "rrr": ("rrr", "ret_r", "adv_r"), "rll": ("rll", "ret_l", "adv_l")}


def md2md_rows(res, geometry, ksc, E, qidx=None, pc=None):
    """Rows of the mode-to-mode files of write_md2md
    (negf/write_data.f90:177-241) for every point of a run with
    ``md2md=True``: {direction: [(q, rows)] per point}, a row (count1,
    count2, omega, k_f(3), k_b(3), kpc_f(3), kpc_b(3), v_f(3), v_b(3), ts,
    tns, i, j) for every pair of propagating modes, j over the column
    problem (outer loop) and i over the row problem, count2 counting the
    columns and count1 every pair; |M_ij|^2 goes to ts when the in-plane k
    of the two modes agree within 1e-5 (squared), else to tns.  Mode order
    as in ``mode_rows``."""
    ksc = np.atleast_2d(np.asarray(ksc, dtype=np.float64))
    E = np.asarray(E, dtype=np.float64)
    npts = E.size
    q_of = np.zeros(npts, dtype=np.int64) if qidx is None else np.asarray(qidx, dtype=np.int64)
    labk = [geometry.label_k(k) for k in ksc]
    pcs = (pc, pc) if pc is None or not isinstance(pc, (tuple, list)) else tuple(pc)
    pcol = _pc_columns(res, labk, q_of, E, pcs, KINDS)
    out = {d: [] for d in MD2MD_FILES}
    for p in range(npts):
        q = int(q_of[p])
        lk = labk[q]
        w = float(np.sqrt(E[p]))
        for d, (mat, kf_kind, kb_kind) in MD2MD_FILES.items():
            M = res["md2md"][p, MATRICES.index(mat)]
            kf, kb = _mode_k(res, p, kf_kind, lk), _mode_k(res, p, kb_kind, lk)
            pf_, pb = pcol[kf_kind][p], pcol[kb_kind][p]
            rows, c1, c2 = [], 0, 0
            for j in range(kb.shape[0]):
                if kb[j, 2] >= 99.9:
                    continue
                c2 += 1
                for i in range(kf.shape[0]):
                    if kf[i, 2] >= 99.9:
                        continue
                    c1 += 1
                    dk = kf[i, :2] - kb[j, :2]
                    v = float(M[i, j])
                    ts, tns = (v, 0.0) if float(dk @ dk) < 1.0e-5 else (0.0, v)
                    rows.append((c1, c2, w, *kf[i], *kb[j], *pf_[i, :3], *pb[j, :3], *pf_[i, 3:], *pb[j, 3:],
                                 ts, tns, i + 1, j + 1))
            out[d].append((q, rows))
    return out


def mode_rows(res, geometry, ksc, E, qidx=None, pc=None):
    """Rows of the per-k mode files for every point of a per-mode run.

    res: transport_tdb_modes(..., per_mode=True); ksc (nq, 3); E (npts,)
    energies (omega^2).  Returns {file name: [(q, rows)] per point}, rows a
    list of tuples (count, omega, k(3), k_pc(3), v_pc(3), sums...) as
    write_specular (sums r_s, r_t, r_s/r_t) and write_md (sums r_s, r_t,
    t_s, t_t) write them (negf/write_data.f90:3-176): one row per
    propagating incoming mode, r_t the sum of |M_ji|^2 over the propagating
    outgoing modes j and r_s over those whose in-plane k is within 1e-5
    (squared) of the incoming mode's.  The primitive-cell k and velocity
    columns (find_k_pc, velocity_mat.f90:2370-2383) come from ``pc``, an
    ``unfold_pc.PrimitiveCell`` (both leads) or a (left, right) pair, and
    are zero without it.  Rows follow this library's mode order, which can
    differ from LAPACK's inside an energy."""
    ksc = np.atleast_2d(np.asarray(ksc, dtype=np.float64))
    E = np.asarray(E, dtype=np.float64)
    npts = E.size
    q_of = np.zeros(npts, dtype=np.int64) if qidx is None else np.asarray(qidx, dtype=np.int64)
    nl, nr = res["nl"], res["nr"]
    size = {"adv_l": nl, "ret_l": nl, "ret_r": nr, "adv_r": nr}
    labk = [geometry.label_k(k) for k in ksc]
    out = {name: [] for name in MODE_FILES}
    pcs = (pc, pc) if pc is None or not isinstance(pc, (tuple, list)) else tuple(pc)
    # primitive-cell columns of the incoming modes of every point, one batch per side
    pcol = {}
    for kind, side in (("adv_l", 0), ("adv_r", 1)):
        ki = KINDS.index(kind)
        cols = np.zeros((npts, size[kind], 6))
        if pcs[side] is not None:
            kz, bz = res["mode_kz"][:, ki, :size[kind]], res["mode_bz"][:, ki, :size[kind]]
            pp, ii = np.nonzero((kz < 99.9) & (bz > 0))
            if pp.size:
                lk = np.array([labk[int(q_of[a])][bz[a, i] - 1] for a, i in zip(pp, ii)])
                lk[:, 2] = kz[pp, ii]
                kp, vp = pcs[side].unfold(E[pp], lk)
                cols[pp, ii, :3], cols[pp, ii, 3:] = kp, vp
        pcol[kind] = cols
    for p in range(npts):
        q = int(q_of[p])
        lk = labk[q]
        w = float(np.sqrt(E[p]))

        def kvec(kind):
            ki = KINDS.index(kind)
            kz, bz = res["mode_kz"][p, ki], res["mode_bz"][p, ki]
            k = np.full((size[kind], 3), 100.0)
            for i in range(size[kind]):
                if kz[i] < 99.9 and bz[i] > 0:
                    k[i] = lk[bz[i] - 1]
                    k[i, 2] = kz[i]
            return k

        def sums(mat, kb, i):
            S = res["col_sums"][p, MATRICES.index(mat), i]
            tot = float(np.sum(S))
            d = lk[:, :2] - kb[i, :2]
            spec = float(np.sum(S[np.einsum("ij,ij->i", d, d) < 1.0e-5]))
            return _clamp(spec), _clamp(tot)

        inc = {kind: (kvec(kind), pcol[kind][p]) for kind in ("adv_l", "adv_r")}
        for name, (mat, kind) in SPECULAR_FILES.items():
            kb, pcols = inc[kind]
            rows, c = [], 0
            for i in range(size[kind]):
                if kb[i, 2] < 99.9:
                    c += 1
                    rs, rt = sums(mat, kb, i)
                    rows.append((c, w, *kb[i], *pcols[i], rs, rt, rs / rt if rt != 0.0 else 0.0))
            out[name].append((q, rows))
        for name, (tmat, rmat, kind) in MD_FILES.items():
            kb, pcols = inc[kind]
            rows, c = [], 0
            for i in range(size[kind]):
                if kb[i, 2] < 99.9:
                    c += 1
                    rs, rt = sums(rmat, kb, i)
                    ts, tt = sums(tmat, kb, i)
                    rows.append((c, w, *kb[i], *pcols[i], rs, rt, ts, tt))
            out[name].append((q, rows))
    return out
