"""Host-side mirror of the reference's transport interface over the C ABI.

The reference drives, for every (ie, ik) of its shard,

    call surface_green_tdb_mpi(ie, ik, gl_adv, gr_ret, ..., Egrid, Haml, Hamr, Hamlv, Hamrv)
    call get_G_full_tdb_mpi(ie, ik, ..., transl_reduce, transr_reduce, ..., hamd, hamdv, hamld, hamrd, haml, hamr)

(negf/phinfortran.f90:1196-1213).  ``transport_tdb`` takes the same blocks
(as numpy complex128 arrays, one set per q) and the same physics parameters,
and returns transl/transr for the whole batch of points in one call of the
fused GPU kernel.  Errors follow the reference's behaviour of stopping on a
singular or non-finite block (negf/util.f90:29-66): a PFError is raised,
unless ``check=False`` in which case the per-point status words are returned.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi

# Block order of the C ABI.
BLOCK_NAMES = ("HL", "HLv", "HR", "HRv", "Hd", "Hdv", "Hld", "Hrd")

PF_STATUS_SINGULAR = 1
PF_STATUS_NAN = 2
PF_STATUS_NOT_CONVERGED = 4


def fortran_block(a):
    """(..., rows, cols) complex -> float64 buffer in column-major block order."""
    a = np.asarray(a, dtype=np.complex128)
    return np.ascontiguousarray(np.swapaxes(a, -1, -2)).view(np.float64)


@dataclass
class TdbBlocks:
    """tdb block set; each array either (m, k) for one q or (nq, m, k)."""
    HL: np.ndarray
    HLv: np.ndarray
    HR: np.ndarray
    HRv: np.ndarray
    Hd: np.ndarray    # (L, n, n) or (nq, L, n, n)
    Hdv: np.ndarray   # (L-1, n, n) or (nq, L-1, n, n)
    Hld: np.ndarray
    Hrd: np.ndarray

    @classmethod
    def from_dict(cls, d):
        return cls(**{k: d[k] for k in BLOCK_NAMES})

    def stacked(self):
        """Return (nq, dims, dict of stacked arrays with a leading q axis)."""
        Hd = np.asarray(self.Hd)
        if Hd.ndim == 3:
            arrs = {k: np.asarray(getattr(self, k))[None] for k in BLOCK_NAMES}
        else:
            arrs = {k: np.asarray(getattr(self, k)) for k in BLOCK_NAMES}
        nq, L, n, _ = arrs["Hd"].shape
        nl = arrs["HL"].shape[-1]
        nr = arrs["HR"].shape[-1]
        if arrs["Hdv"].size == 0:
            arrs["Hdv"] = np.zeros((nq, 0, n, n), np.complex128)
        _check_shapes(arrs, nq, L, n, nl, nr)
        return nq, (n, nl, nr, L), arrs


def _check_shapes(a, nq, L, n, nl, nr):
    want = {"HL": (nq, nl, nl), "HLv": (nq, nl, nl), "HR": (nq, nr, nr), "HRv": (nq, nr, nr),
            "Hd": (nq, L, n, n), "Hdv": (nq, max(L - 1, 0), n, n), "Hld": (nq, nl, n),
            "Hrd": (nq, nr, n)}
    for k, shp in want.items():
        if tuple(a[k].shape) != shp:
            raise ValueError(f"block {k}: shape {a[k].shape}, expected {shp}")


def _ptr(a, ctype=C.c_double):
    return a.ctypes.data_as(C.POINTER(ctype))


NMAX_RESIDENT = 48   # PF_NMAX_RESIDENT
# precision -> arith of the large-block entry (PF_ARITH_FP64 / _DF64 / _TC)
TILED_ARITH = {"fp64": 0, "df64": 1, "tc": 2, "mixed": 2}


def _circular_args(circular, nl, nr):
    """(n_bloch_y, n_bloch_x, gr[4]) of the block-circulant lead option."""
    if isinstance(circular, dict):
        ny, nx, gr = circular["n_bloch_y"], circular["n_bloch_x"], circular["gr"]
    else:
        ny, nx, gr = circular
    gr = np.ascontiguousarray(np.broadcast_to(np.asarray(gr, dtype=np.float64), (4,)))
    ny, nx = int(ny), int(nx)
    if ny < 1 or nx < 1 or nl != nr or nl % (ny * nx):
        raise ValueError("block-circulant leads need nl == nr, a multiple of n_bloch_y * n_bloch_x")
    return ny, nx, gr


def _transport_tiled(E, nq, dims, arrs, *, eta, eta0, convergence, dev_factor, qidx, zero_flag, max_iter,
                     want_transr, check, precision, circular=None):
    """Blocks above the resident size: pf_transport_tdb_tiled_dev on torch
    device buffers (T_L only).  precision: "fp64" (SIMT FP64 block
    products), "tc" (the FP64 algorithm with every block product on the
    tensor cores as exact BF16 slice products), "df64" (double-float
    arithmetic on the FP32 pipe, ~48-bit); "mixed" selects "tc".
    circular: block-circulant leads; want_transr: T_R from the right-to-left
    sweep as well (both through pf_transport_tdb_tiled_ex_dev)."""
    import torch
    arith = TILED_ARITH[precision]
    lib = _abi.load()
    n, nl, nr, L = dims
    dev = {k: torch.from_numpy(fortran_block(v).copy()).cuda() for k, v in arrs.items()}
    E = np.ascontiguousarray(E, dtype=np.float64)
    npts = E.size
    Ed = torch.from_numpy(E).cuda()
    qd = None if qidx is None else torch.from_numpy(np.ascontiguousarray(qidx, dtype=np.int32)).cuda()
    zd = None if zero_flag is None else torch.from_numpy(np.ascontiguousarray(zero_flag, dtype=np.int32)).cuda()
    tl = torch.zeros(max(npts, 1), dtype=torch.float64, device="cuda")
    trr = torch.zeros(max(npts, 1), dtype=torch.float64, device="cuda") if want_transr else None
    st = torch.zeros(max(npts, 1), dtype=torch.int32, device="cuda")
    it = torch.zeros((max(npts, 1), 2), dtype=torch.int32, device="cuda")
    p = lambda t: None if t is None else t.data_ptr()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    head = (n, nl, nr, L, nq, *[dev[k].data_ptr() for k in BLOCK_NAMES], npts, Ed.data_ptr(), p(qd), p(zd), eta,
            eta0, dev_factor, convergence, max_iter, arith)
    outs = (tl.data_ptr(), st.data_ptr(), it.data_ptr())
    if circular is None and not want_transr:
        ws = lib.pf_transport_tdb_tiled_workspace_size(n, nl, nr, L, nq, npts, arith)
        if ws == 0:
            _abi.check(-3)
        work = torch.empty(ws, dtype=torch.uint8, device="cuda")
        rc = lib.pf_transport_tdb_tiled_dev(*head, *outs, work.data_ptr(), ws, stream)
    else:
        # pf_transport_tdb_tiled_ex_dev: block-circulant leads and / or T_R
        ny, nx, gr = _circular_args(circular, nl, nr) if circular is not None else (1, 1, None)
        ws = lib.pf_transport_tdb_tiled_ex_workspace_size(n, nl, nr, L, nq, npts, arith, ny, nx)
        if ws == 0:
            _abi.check(-3)
        work = torch.empty(ws, dtype=torch.uint8, device="cuda")
        rc = lib.pf_transport_tdb_tiled_ex_dev(*head, ny, nx, None if gr is None else _ptr(gr), tl.data_ptr(),
                                               p(trr), st.data_ptr(), it.data_ptr(), work.data_ptr(), ws, stream)
    if rc != 0:
        raise _abi.PFError(rc, lib.pf_tiled_last_error().decode(errors="replace"))
    torch.cuda.synchronize()
    status = st.cpu().numpy()[:npts]
    if check and (status != 0).any():
        raise _abi.PFError(-4, f"point status flags 0x{int(np.bitwise_or.reduce(status)):x}")
    return dict(transl=tl.cpu().numpy()[:npts], transr=None if trr is None else trr.cpu().numpy()[:npts],
                status=status, iters=it.cpu().numpy()[:npts])


def transport_tdb(E, blocks, *, eta, eta0, convergence, dev_factor=10.0, qidx=None,
                  zero_flag=None, max_iter=1000, want_transr=True, check=True,
                  precision="fp64", refine_iters=2, circular=None):
    """Transmission for a batch of points through the host-pointer C entry.

    E: (npts,) energies (omega^2 for phonons).  blocks: TdbBlocks or dict.
    qidx: (npts,) q index into the stacked blocks (None: all 0).
    zero_flag: (npts,) nonzero -> T forced to 0 (the reference's ie == 1).
    precision: "fp64" (pf_transport_tdb) or "mixed" (pf_transport_tdb_mixed:
    FP64-grade lead decimations with their block products on the tensor
    cores, FP32 factorisation, double-float refinement: one sweep for every
    point and up to `refine_iters` - 1 more for the points whose last
    correction of G_{0,N+1} was above 3e-5 relative; T_L only).
    Blocks above 48 go through the large-block entry, where "mixed" (or
    "tc") puts the block products on the tensor cores and "df64" selects
    the double-float engine.
    circular: block-circulant leads (the reference's circular_flag = 1),
    (n_bloch_y, n_bloch_x, gr) or a dict with those keys, gr = the G.R
    products {left y, left x, right y, right x}; the lead surface Green's
    functions then come from circular_g (negf/circular.f90:42-105) on the
    large-block engine, at any block size.  On the large-block engine
    want_transr adds the right-to-left sweep and T_R (off in "mixed" below
    48, which computes T_L only).
    Returns dict(transl, transr, status, iters).
    """
    if precision not in TILED_ARITH:
        raise ValueError("precision must be 'fp64', 'mixed', 'tc' or 'df64'")
    lib = _abi.load()
    if isinstance(blocks, dict):
        blocks = TdbBlocks.from_dict(blocks)
    nq, (n, nl, nr, L), arrs = blocks.stacked()
    if max(n, nl, nr) <= NMAX_RESIDENT and precision in ("tc", "df64") and circular is None:
        raise ValueError("precision 'tc' and 'df64' are large-block (n > 48) arithmetics")
    if max(n, nl, nr) > NMAX_RESIDENT or circular is not None:
        return _transport_tiled(E, nq, (n, nl, nr, L), arrs, eta=eta, eta0=eta0, convergence=convergence,
                                dev_factor=dev_factor, qidx=qidx, zero_flag=zero_flag, max_iter=max_iter,
                                want_transr=want_transr, check=check, precision=precision, circular=circular)
    buf = {k: fortran_block(v) for k, v in arrs.items()}
    E = np.ascontiguousarray(E, dtype=np.float64)
    npts = E.shape[0]
    q = None if qidx is None else np.ascontiguousarray(qidx, dtype=np.int32)
    z = None if zero_flag is None else np.ascontiguousarray(zero_flag, dtype=np.int32)
    if q is not None and (q.shape != (npts,) or q.min(initial=0) < 0 or q.max(initial=0) >= nq):
        raise ValueError("qidx out of range")
    tl = np.zeros(npts)
    tr = np.zeros(npts)
    st = np.zeros(npts, dtype=np.int32)
    it = np.zeros((npts, 2), dtype=np.int32)
    qp = None if q is None else _ptr(q, C.c_int)
    zp = None if z is None else _ptr(z, C.c_int)
    if precision == "fp64":
        rc = lib.pf_transport_tdb(n, nl, nr, L, nq, *[_ptr(buf[k]) for k in BLOCK_NAMES], npts, _ptr(E),
                                  qp, zp, eta, eta0, dev_factor, convergence, max_iter, int(bool(want_transr)),
                                  _ptr(tl), _ptr(tr), _ptr(st, C.c_int), _ptr(it, C.c_int))
    else:
        want_transr = False
        rc = lib.pf_transport_tdb_mixed(n, nl, nr, L, nq, *[_ptr(buf[k]) for k in BLOCK_NAMES], npts, _ptr(E),
                                        qp, zp, eta, eta0, dev_factor, convergence, max_iter, int(refine_iters),
                                        _ptr(tl), _ptr(st, C.c_int), _ptr(it, C.c_int))
    if rc != 0 and (check or rc != -4):
        _abi.check(rc)
    return dict(transl=tl, transr=tr if want_transr else None, status=st, iters=it)


class DeviceTransport:
    """Blocks resident in HBM (torch tensors used only as device buffers).

    ``run`` launches the fused kernel on device-resident energies and writes
    device-resident outputs: this is the path the throughput benchmark
    times.  The work queue, scratch and outputs are allocated once.
    """

    def __init__(self, blocks, npts_max, *, eta, eta0, convergence, dev_factor=10.0,
                 max_iter=1000, want_transr=False, device="cuda", precision="fp64", refine_iters=2,
                 lead_arith="auto"):
        import torch
        if isinstance(blocks, dict):
            blocks = TdbBlocks.from_dict(blocks)
        nq, (n, nl, nr, L), arrs = blocks.stacked()
        dev = {k: torch.from_numpy(fortran_block(v).copy()).to(device) for k, v in arrs.items()}
        self._setup(dev, (n, nl, nr, L, nq), npts_max, eta=eta, eta0=eta0, convergence=convergence,
                    dev_factor=dev_factor, max_iter=max_iter, want_transr=want_transr, device=device,
                    precision=precision, refine_iters=refine_iters, lead_arith=lead_arith)

    @classmethod
    def from_device(cls, dev, dims, npts_max, **kw):
        """Blocks already on the device: dev maps the block names to float64
        buffers in the C ABI's layout ([q][block][col][row] interleaved
        complex), dims = (n, nl, nr, L, nq)."""
        obj = cls.__new__(cls)
        obj._setup(dev, tuple(dims), npts_max, **kw)
        return obj

    def _setup(self, dev, dims, npts_max, *, eta, eta0, convergence, dev_factor=10.0, max_iter=1000,
               want_transr=False, device="cuda", precision="fp64", refine_iters=2, lead_arith="auto"):
        import torch
        self.torch = torch
        lib = _abi.load()
        n, nl, nr, L, nq = dims
        self.dims = dims
        self.dev = dev
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.precision = precision
        self.refine_iters = int(refine_iters)
        # lead decimations of the mixed path: PF_ARITH_AUTO (default: FP64 with
        # tensor-core products up to 32, double-float above), PF_ARITH_FP64,
        # PF_ARITH_SPLIT (first steps FP64, the rest double-float) or PF_ARITH_DF64
        lead_codes = {"auto": -1, "split": 3, "fp64": 0, "df64": 1}
        if lead_arith not in lead_codes:
            raise ValueError("lead_arith must be 'auto', 'split', 'fp64' or 'df64'")
        self.lead_arith = lead_codes[lead_arith]
        if precision == "mixed":
            want_transr = False
        self.params = (eta, eta0, dev_factor, convergence, max_iter, int(bool(want_transr)))
        self.npts_max = npts_max
        if precision == "fp64":
            ws = lib.pf_transport_tdb_workspace_size(n, nl, nr, nq, npts_max)
        else:
            ws = lib.pf_transport_tdb_mixed_workspace_size(n, nl, nr, L, nq, npts_max)
        if ws == 0:
            _abi.check(-3)
        self.work = torch.empty(ws, dtype=torch.uint8, device=device)
        self.transl = torch.zeros(npts_max, dtype=torch.float64, device=device)
        self.transr = torch.zeros(npts_max, dtype=torch.float64, device=device)
        self.status = torch.zeros(npts_max, dtype=torch.int32, device=device)
        self.iters = torch.zeros((npts_max, 2), dtype=torch.int32, device=device)

    def capture(self, E, qidx=None, zero_flag=None):
        """Record one ``run`` on these device-resident inputs into a CUDA
        graph and return it (``g.replay()`` re-runs the whole batched pass --
        block conversions, lead decimations, factorisation, refinement
        sweeps, Caroli traces -- with no host work; the outputs land in
        ``transl`` / ``status`` / ``iters`` as after ``run``).  The C entry
        is stream-ordered with no host synchronisation, so it captures as is;
        one uncaptured run first sets the kernels' attributes."""
        torch = self.torch
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self.run(E, qidx, zero_flag, stream=side)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="thread_local"):
            self.run(E, qidx, zero_flag, stream=torch.cuda.current_stream())
        return g

    def run(self, E, qidx=None, zero_flag=None, stream=None):
        torch = self.torch
        lib = _abi.load()
        n, nl, nr, L, nq = self.dims
        npts = int(E.shape[0])
        if npts > self.npts_max:
            raise ValueError("more points than allocated")
        s = stream if stream is not None else torch.cuda.current_stream()
        eta, eta0, dev_factor, conv, max_iter, want_transr = self.params
        d = self.dev
        qp = None if qidx is None else qidx.data_ptr()
        zp = None if zero_flag is None else zero_flag.data_ptr()
        if self.precision == "fp64":
            rc = lib.pf_transport_tdb_dev(
                n, nl, nr, L, nq, *[d[k].data_ptr() for k in BLOCK_NAMES], npts, E.data_ptr(), qp, zp,
                eta, eta0, dev_factor, conv, max_iter, want_transr,
                self.transl.data_ptr(), self.transr.data_ptr(), self.status.data_ptr(), self.iters.data_ptr(),
                self.work.data_ptr(), self.work.numel(), C.c_void_p(s.cuda_stream))
        else:
            rc = lib.pf_transport_tdb_mixed_ex_dev(
                n, nl, nr, L, nq, *[d[k].data_ptr() for k in BLOCK_NAMES], npts, E.data_ptr(), qp, zp,
                eta, eta0, dev_factor, conv, max_iter, self.refine_iters, self.lead_arith,
                self.transl.data_ptr(), self.status.data_ptr(), self.iters.data_ptr(),
                self.work.data_ptr(), self.work.numel(), C.c_void_p(s.cuda_stream))
        _abi.check(rc)
        return self.transl[:npts], self.transr[:npts], self.status[:npts]
