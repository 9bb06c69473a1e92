"""The tensor-core complex GEMM (pf_tc_zgemm_dev) against numpy complex128.

Integer-valued inputs must come out exact (the slice products are summed
exactly); random inputs must match FP64 to the normwise FP64 bound
|C - C64| <= k 2^-50 |A| |B| (the split keeps 56 bits); rows scaled across
hundreds of orders of magnitude keep their relative accuracy; a NaN entry
makes its output row NaN.
"""
import ctypes as C

import numpy as np
import pytest

from phinfortran_gb300 import _abi

pytestmark = pytest.mark.gpu


def _run(A, B, Cin, transa, transb, alpha, beta, shared_a=False):
    """A, B, Cin: numpy complex arrays [batch][rows][cols] (C order per
    matrix, converted to column-major here)."""
    import torch
    lib = _abi.load()
    batch = Cin.shape[0]
    m, n = Cin.shape[1], Cin.shape[2]
    k = A.shape[2] if transa == "N" else A.shape[1]

    def dev(X):
        f = np.ascontiguousarray(np.transpose(X, (0, 2, 1)))   # column-major per matrix
        return torch.from_numpy(f.view(np.float64).reshape(-1).copy()).cuda()
    dA, dB, dC = dev(A), dev(B), dev(Cin)
    lda, ldb, ldc = A.shape[1], B.shape[1], m
    sA = 0 if shared_a else A.shape[1] * A.shape[2]
    sB, sC = B.shape[1] * B.shape[2], m * n
    ws = lib.pf_tc_zgemm_workspace_size(m, n, k, batch, int(shared_a), 0)
    work = torch.empty(ws, dtype=torch.uint8, device="cuda")
    rc = lib.pf_tc_zgemm_dev(ord(transa), ord(transb), m, n, k, alpha, dA.data_ptr(), lda, sA, dB.data_ptr(), ldb,
                             sB, beta, dC.data_ptr(), ldc, sC, batch, work.data_ptr(), ws,
                             C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc != 0:
        raise _abi.PFError(rc, lib.pf_tc_last_error().decode())
    out = dC.cpu().numpy().view(np.complex128).reshape(batch, n, m)
    return np.transpose(out, (0, 2, 1))


def _ref(A, B, Cin, transa, transb, alpha, beta):
    opA = A if transa == "N" else np.conj(np.transpose(A, (0, 2, 1)))
    opB = B if transb == "N" else np.conj(np.transpose(B, (0, 2, 1)))
    return alpha * (opA @ opB) + beta * Cin, np.abs(opA) @ np.abs(opB)


def _cplx(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def test_integer_inputs_are_exact(cuda_ready):
    rng = np.random.default_rng(1)
    A = rng.integers(-1000, 1001, (2, 37, 71)) + 1j * rng.integers(-1000, 1001, (2, 37, 71))
    B = rng.integers(-1000, 1001, (2, 71, 53)) + 1j * rng.integers(-1000, 1001, (2, 71, 53))
    Cin = np.zeros((2, 37, 53), complex)
    out = _run(A, B, Cin, "N", "N", 1.0, 0.0)
    ref, _ = _ref(A, B, Cin, "N", "N", 1.0, 0.0)
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("m,n,k,ta,tb", [(96, 96, 96, "N", "N"), (216, 216, 216, "N", "N"), (48, 200, 300, "C", "N"),
                                         (129, 65, 1, "N", "C"), (64, 64, 640, "C", "C"), (384, 96, 384, "N", "N")])
def test_random_matches_fp64_bound(cuda_ready, m, n, k, ta, tb):
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    batch = 3
    A = _cplx(rng, batch, *((m, k) if ta == "N" else (k, m)))
    B = _cplx(rng, batch, *((k, n) if tb == "N" else (n, k)))
    Cin = _cplx(rng, batch, m, n)
    out = _run(A, B, Cin, ta, tb, 2.0, -0.5)
    ref, mag = _ref(A, B, Cin, ta, tb, 2.0, -0.5)
    bound = k * 2.0 ** -50 * (2.0 * mag + 0.5 * np.abs(Cin)) + 1e-300
    assert (np.abs(out - ref) <= bound).all(), float((np.abs(out - ref) / bound).max())


def test_shared_operand_and_scaled_rows(cuda_ready):
    rng = np.random.default_rng(5)
    m, n, k, batch = 40, 33, 90, 4
    A = _cplx(rng, 1, m, k) * np.logspace(-150, 150, m)[None, :, None]
    A = np.repeat(A, batch, axis=0)
    B = _cplx(rng, batch, k, n)
    Cin = np.zeros((batch, m, n), complex)
    out = _run(A[:1], B, Cin, "N", "N", 1.0, 0.0, shared_a=True)
    ref, mag = _ref(A, B, Cin, "N", "N", 1.0, 0.0)
    rel = np.abs(out - ref) / mag
    assert rel.max() < k * 2.0 ** -50


def test_nan_row_propagates(cuda_ready):
    rng = np.random.default_rng(6)
    A = _cplx(rng, 1, 20, 30)
    A[0, 7, 11] = np.nan
    B = _cplx(rng, 1, 30, 10)
    out = _run(A, B, np.zeros((1, 20, 10), complex), "N", "N", 1.0, 0.0)
    assert np.isnan(out[0, 7]).all()
    assert np.isfinite(np.delete(out[0], 7, axis=0)).all()
