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
ARITH = {"fp64": 0, "df64": 1}   # PF_ARITH_FP64, PF_ARITH_DF64


def _unpack(buf, shape):
    """Column-major interleaved complex device buffer -> numpy (.., rows, cols)."""
    z = buf.cpu().numpy().view(np.complex128)[:int(np.prod(shape))]
    *lead, r, c = shape
    return z.reshape(tuple(lead) + (c, r)).swapaxes(-1, -2)


class DeviceGradient:
    """Blocks, accumulators and scratch resident in HBM for repeated adjoint
    launches; ``run`` takes device-resident energies and weights."""

    def __init__(self, blocks, npts_max, *, eta, eta0, convergence, dev_factor=10.0, max_iter=1000,
                 ckpt=0, arith="fp64", device="cuda"):
        import torch
        self.torch = torch
        lib = _abi.load()
        if isinstance(blocks, dict):
            blocks = TdbBlocks.from_dict(blocks)
        nq, (n, nl, nr, L), arrs = blocks.stacked()
        self.dims = (n, nl, nr, L, nq)
        self.dev = {k: torch.from_numpy(fortran_block(v).copy()).to(device) for k, v in arrs.items()}
        self.params = (eta, eta0, dev_factor, convergence, max_iter)
        self.ckpt = int(ckpt)
        if arith not in ARITH:
            raise ValueError(f"arith must be one of {sorted(ARITH)}")
        self.arith = ARITH[arith]
        self.npts_max = npts_max
        self.shapes = dict(Hd=(nq, L, n, n), Hdv=(nq, max(L - 1, 0), n, n), Hld=(nq, n, nl), Hrd=(nq, n, nr))
        self.g = {k: torch.zeros(max(2 * int(np.prod(s)), 2), dtype=torch.float64, device=device)
                  for k, s in self.shapes.items()}
        ws = lib.pf_transport_tdb_grad_workspace_size(n, nl, nr, L, nq, npts_max, self.ckpt, self.arith)
        if ws == 0:
            raise _abi.PFError(-3, "gradient kernel does not fit (block size > 48?)")
        self.work = torch.empty(ws, dtype=torch.uint8, device=device)
        self.transl = torch.zeros(npts_max, dtype=torch.float64, device=device)
        self.status = torch.zeros(npts_max, dtype=torch.int32, device=device)
        self.iters = torch.zeros((npts_max, 2), dtype=torch.int32, device=device)

    def run(self, E, weights=None, qidx=None, zero_flag=None, stream=None):
        torch = self.torch
        lib = _abi.load()
        n, nl, nr, L, nq = self.dims
        npts = int(E.shape[0])
        if npts > self.npts_max:
            raise ValueError("more points than allocated")
        s = stream if stream is not None else torch.cuda.current_stream()
        eta, eta0, dev_factor, conv, max_iter = self.params
        p = lambda t: None if t is None else t.data_ptr()
        g = self.g
        rc = lib.pf_transport_tdb_grad_dev(n, nl, nr, L, nq, *[self.dev[k].data_ptr() for k in BLOCK_NAMES],
                                           npts, E.data_ptr(), p(qidx), p(zero_flag), p(weights), eta, eta0,
                                           dev_factor, conv, max_iter, self.ckpt, self.arith,
                                           self.transl.data_ptr(),
                                           self.status.data_ptr(), self.iters.data_ptr(), g["Hd"].data_ptr(),
                                           g["Hdv"].data_ptr() if L > 1 else None, g["Hld"].data_ptr(),
                                           g["Hrd"].data_ptr(), self.work.data_ptr(), self.work.numel(),
                                           C.c_void_p(s.cuda_stream))
        if rc != 0:
            raise _abi.PFError(rc, lib.pf_grad_last_error().decode(errors="replace"))
        return self.transl[:npts], self.status[:npts]

    def sensitivities(self):
        """M dict (leading q axis) as numpy, after the stream has finished."""
        return {k: _unpack(self.g[k], s) for k, s in self.shapes.items()}


def transport_grad(E, blocks, weights=None, *, eta, eta0, convergence, dev_factor=10.0, qidx=None,
                   zero_flag=None, max_iter=1000, ckpt=0, arith="fp64", check=True):
    """Forward T (npts,) and M dict (leading q axis) through the adjoint kernel."""
    import torch
    E = np.ascontiguousarray(E, dtype=np.float64)
    dg = DeviceGradient(blocks, max(E.size, 1), eta=eta, eta0=eta0, convergence=convergence,
                        dev_factor=dev_factor, max_iter=max_iter, ckpt=ckpt, arith=arith)
    dev = lambda a, dt: None if a is None else torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).cuda()
    tl, st = dg.run(dev(E, np.float64), dev(weights, np.float64), dev(qidx, np.int32), dev(zero_flag, np.int32))
    torch.cuda.synchronize()
    status = st.cpu().numpy()
    if check and (status != 0).any():
        raise _abi.PFError(-4, f"point status flags 0x{int(np.bitwise_or.reduce(status)):x}")
    return tl.cpu().numpy(), dg.sensitivities(), status


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

        forward(masses, springs, bar, omega, temperature, params, precision, grad_arith, ckpt)
        precision: forward path ("fp64" or "mixed"); grad_arith: "fp64" or
        "df64" for the adjoint; ckpt: checkpoint interval (0 = sqrt(L+2)).
        """

        @staticmethod
        def forward(ctx, masses, springs, bar, omega, temperature, params, precision="fp64", grad_arith="df64",
                    ckpt=0):
            from .transport import transport_tdb
            m = masses.detach().cpu().numpy().astype(np.float64)
            k = springs.detach().cpu().numpy().astype(np.float64)
            blocks = bar.blocks(m, k)
            E = np.asarray(omega, dtype=np.float64) ** 2
            wts = landauer_weights(omega, temperature)
            r = transport_tdb(E, blocks, want_transr=False, precision=precision, **params)
            ctx.save_for_backward(masses, springs)
            ctx.bar, ctx.E, ctx.wts, ctx.params = bar, E, wts, params
            ctx.grad_arith, ctx.ckpt = grad_arith, ckpt
            return torch.tensor(float(np.dot(wts, r["transl"])), dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad_out):
            masses, springs = ctx.saved_tensors
            m = masses.detach().cpu().numpy().astype(np.float64)
            k = springs.detach().cpu().numpy().astype(np.float64)
            blocks = ctx.bar.blocks(m, k)
            _, M, _ = transport_grad(ctx.E, blocks, ctx.wts, ckpt=ctx.ckpt, arith=ctx.grad_arith, **ctx.params)
            GD = ctx.bar.sensitivity_matrix({kk: v[0] for kk, v in M.items()})
            gm, gk = ctx.bar.parameter_gradient(GD, m, k)
            g = float(grad_out)
            return (torch.from_numpy(gm * g).to(masses), torch.from_numpy(gk * g).to(springs),
                    None, None, None, None, None, None, None)

    return ConductanceFunction


def conductance_fn():
    """The torch.autograd.Function class (built lazily so torch stays optional)."""
    return _torch_function()
