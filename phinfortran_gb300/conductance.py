"""Landauer conductance of T(omega) over the C ABI (pf_landauer_conductance).

Mirrors examples/negf/si-si/condt.py: ``conductance(E, trans_k, temps, area)``
takes the reference's omega^2 grid (THz^2) and the (ne, nk) transmission
table of transl_tot.dat, averages over k and integrates on the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi

THZ2RADS = 1e12 * np.pi * 2


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def conductance(E, trans, temps, area):
    lib = _abi.load()
    trans = np.asarray(trans, dtype=np.float64)
    if trans.ndim == 2:                       # (ne, nk): k average as condt.py:44-51
        trans = trans.sum(axis=1) / trans.shape[1]
    w = np.ascontiguousarray(np.sqrt(np.asarray(E, dtype=np.float64)) * THZ2RADS)
    tr = np.ascontiguousarray(trans)
    T = np.ascontiguousarray(np.atleast_1d(np.asarray(temps, dtype=np.float64)))
    out = np.zeros(T.size)
    rc = lib.pf_landauer_conductance(w.size, _ptr(w), _ptr(tr), T.size, _ptr(T), float(area), _ptr(out))
    if rc != 0:
        raise _abi.PFError(rc, lib.pf_cond_last_error().decode(errors="replace"))
    return out
