"""ctypes wrapper of the C restatement of the transmission oracle
(oracle/negf_c.c; test infrastructure and the CPU baseline of bench.py).
``transport_c`` gives T_L of a batch of energies of one q, in parallel over
the energies on the host cores, following oracle/negf.py."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_c

_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build_c.build())
        d = C.POINTER(C.c_double)
        lib.oracle_c_transport.restype = C.c_int
        lib.oracle_c_transport.argtypes = [C.c_int] * 4 + [d] * 8 + [C.c_int, d] + [C.c_double] * 4 + \
            [C.c_int, d, C.POINTER(C.c_int)]
        lib.oracle_c_threads.restype = C.c_int
        lib.oracle_c_threads.argtypes = [C.c_int]
        _lib = lib
    return _lib


def _colmajor(a):
    """Column-major interleaved complex128 of every trailing matrix."""
    a = np.asarray(a, dtype=np.complex128)
    return np.ascontiguousarray(np.swapaxes(a, -1, -2)).view(np.float64)


def transport_c(E, blocks, eta, eta0, convergence, dev_factor, max_iter=1_000_000, threads=0):
    """(T_L (npts,), left decimation iterations (npts,), threads used)."""
    lib = load()
    used = lib.oracle_c_threads(int(threads))
    Hd = np.asarray(blocks["Hd"])
    L, n = Hd.shape[0], Hd.shape[-1]
    nl, nr = np.asarray(blocks["HL"]).shape[-1], np.asarray(blocks["HR"]).shape[-1]
    arrs = [_colmajor(blocks[k]) for k in ("HL", "HLv", "HR", "HRv", "Hd")]
    hdv = _colmajor(blocks["Hdv"]) if L > 1 else np.zeros(2)
    arrs += [hdv, _colmajor(blocks["Hld"]), _colmajor(blocks["Hrd"])]
    E = np.ascontiguousarray(E, dtype=np.float64)
    T = np.zeros(E.size)
    it = np.zeros(E.size, dtype=np.int32)
    p = lambda x: x.ctypes.data_as(C.POINTER(C.c_double))
    bad = lib.oracle_c_transport(n, nl, nr, L, *[p(a) for a in arrs], E.size, p(E), eta, eta0, dev_factor,
                                 convergence, int(max_iter), p(T), it.ctypes.data_as(C.POINTER(C.c_int)))
    if bad:
        raise FloatingPointError(f"{bad} points hit a zero pivot")
    return T, it, used
