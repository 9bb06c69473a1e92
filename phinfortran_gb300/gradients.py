"""Derivatives of T(omega) and of the Landauer conductance on the GPU.

``transport_grad`` calls the adjoint C entry (pf_transport_tdb_grad_dev)
for a weighted batch of points and returns the forward T and the block
sensitivities M_B = sum_p w_p dT_p/dB (dF = Re Tr[dB M_B]).
``landauer_weights`` gives the weights w_p = d kappa / d T_p of the
trapezoid conductance of examples/negf/si-si/condt.py:14-30, so that one
adjoint call yields d kappa / dB.  ``ConductanceFunction`` wraps
kappa(masses, springs) of a simple-cubic bar as a torch.autograd.Function
whose backward is the adjoint kernel (the chain rule from the blocks to the
parameters is ScBar.parameter_gradient).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .transport import BLOCK_NAMES, TdbBlocks, fortran_block

KB = 1.380649e-23
HBAR = 1.0545718e-34
THZ2RADS = 1e12 * np.pi * 2


def _unpack(buf, shape):
    """Column-major interleaved complex device buffer -> numpy (.., rows, cols)."""
    z = buf.cpu().numpy().view(np.complex128)
    *lead, r, c = shape
    return z.reshape(tuple(lead) + (c, r)).swapaxes(-1, -2)


def transport_grad(E, blocks, weights=None, *, eta, eta0, convergence, dev_factor=10.0, qidx=None,
                   zero_flag=None, max_iter=1000, check=True):
    """Forward T (npts,) and M dict (leading q axis) through the adjoint kernel."""
    import torch
    lib = _abi.load()
    if isinstance(blocks, dict):
        blocks = TdbBlocks.from_dict(blocks)
    nq, (n, nl, nr, L), arrs = blocks.stacked()
    dev = {k: torch.from_numpy(fortran_block(v).copy()).cuda() for k, v in arrs.items()}
    E = np.ascontiguousarray(E, dtype=np.float64)
    npts = E.size
    Ed = torch.from_numpy(E).cuda()
    wd = None if weights is None else torch.from_numpy(np.ascontiguousarray(weights, dtype=np.float64)).cuda()
    qd = None if qidx is None else torch.from_numpy(np.ascontiguousarray(qidx, dtype=np.int32)).cuda()
    zd = None if zero_flag is None else torch.from_numpy(np.ascontiguousarray(zero_flag, dtype=np.int32)).cuda()
    tl = torch.zeros(npts, dtype=torch.float64, device="cuda")
    st = torch.zeros(npts, dtype=torch.int32, device="cuda")
    it = torch.zeros(2 * npts, dtype=torch.int32, device="cuda")
    shapes = dict(Hd=(nq, L, n, n), Hdv=(nq, max(L - 1, 0), n, n), Hld=(nq, n, nl), Hrd=(nq, n, nr))
    g = {k: torch.zeros(2 * int(np.prod(s)), dtype=torch.float64, device="cuda") for k, s in shapes.items()}
    ws = lib.pf_transport_tdb_grad_workspace_size(n, nl, nr, L, nq, npts)
    if ws == 0:
        raise _abi.PFError(-3, "gradient kernel does not fit (block size > 48?)")
    work = torch.empty(ws, dtype=torch.uint8, device="cuda")
    p = lambda t: None if t is None else t.data_ptr()
    rc = lib.pf_transport_tdb_grad_dev(n, nl, nr, L, nq, *[dev[k].data_ptr() for k in BLOCK_NAMES], npts,
                                       Ed.data_ptr(), p(qd), p(zd), p(wd), eta, eta0, dev_factor, convergence,
                                       max_iter, tl.data_ptr(), st.data_ptr(), it.data_ptr(),
                                       g["Hd"].data_ptr(), g["Hdv"].data_ptr() if L > 1 else None,
                                       g["Hld"].data_ptr(), g["Hrd"].data_ptr(), work.data_ptr(), ws,
                                       C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc != 0:
        raise _abi.PFError(rc, lib.pf_grad_last_error().decode(errors="replace"))
    torch.cuda.synchronize()
    status = st.cpu().numpy()
    if check and (status != 0).any():
        raise _abi.PFError(-4, f"point status flags 0x{int(np.bitwise_or.reduce(status)):x}")
    M = {k: _unpack(g[k], s) for k, s in shapes.items()}
    return tl.cpu().numpy(), M, status


def landauer_weights(omega_thz, temperature, area=1.0):
    """w_p = d kappa / d T_p for kappa = 1/A 1/(2 pi) trapz(hbar w df/dT T(w), w)
    with w = omega_thz * 2 pi 1e12 (condt.py:14-30, 51)."""
    w = np.asarray(omega_thz, dtype=np.float64) * THZ2RADS
    x = HBAR * w / KB / temperature
    expf = np.exp(x)
    dfdw = expf / (expf - 1) ** 2 * HBAR * w / KB / temperature ** 2
    itd_coef = 1 / area / 2 / np.pi * HBAR * w * dfdw
    tw = np.zeros_like(w)
    dw = np.diff(w)
    tw[:-1] += 0.5 * dw
    tw[1:] += 0.5 * dw
    return itd_coef * tw


def _torch_function():
    import torch

    class ConductanceFunction(torch.autograd.Function):
        """kappa(masses, springs) of an ScBar; backward through the adjoint kernel.

        forward(masses, springs, bar, omega, temperature, params, precision)
        """

        @staticmethod
        def forward(ctx, masses, springs, bar, omega, temperature, params, precision="fp64"):
            from .transport import transport_tdb
            m = masses.detach().cpu().numpy().astype(np.float64)
            k = springs.detach().cpu().numpy().astype(np.float64)
            blocks = bar.blocks(m, k)
            E = np.asarray(omega, dtype=np.float64) ** 2
            wts = landauer_weights(omega, temperature)
            r = transport_tdb(E, blocks, want_transr=False, precision=precision, **params)
            ctx.save_for_backward(masses, springs)
            ctx.bar, ctx.E, ctx.wts, ctx.params = bar, E, wts, params
            return torch.tensor(float(np.dot(wts, r["transl"])), dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad_out):
            masses, springs = ctx.saved_tensors
            m = masses.detach().cpu().numpy().astype(np.float64)
            k = springs.detach().cpu().numpy().astype(np.float64)
            blocks = ctx.bar.blocks(m, k)
            _, M, _ = transport_grad(ctx.E, blocks, ctx.wts, **ctx.params)
            GD = ctx.bar.sensitivity_matrix({kk: v[0] for kk, v in M.items()})
            gm, gk = ctx.bar.parameter_gradient(GD, m, k)
            g = float(grad_out)
            return (torch.from_numpy(gm * g).to(masses), torch.from_numpy(gk * g).to(springs),
                    None, None, None, None, None)

    return ConductanceFunction


def conductance_fn():
    """The torch.autograd.Function class (built lazily so torch stays optional)."""
    return _torch_function()
