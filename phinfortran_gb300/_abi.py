"""ctypes binding of the C ABI declared in include/phinfortran_gb300.h.

The shared library is built in-tree by ``phinfortran_gb300.build``.  Loading
fails loudly when it is missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB

_lib = None

# name -> (restype, argtypes), mirroring include/phinfortran_gb300.h
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
SIGNATURES = {
    "pf_last_error": (C.c_char_p, []),
    "pf_version": (C.c_int, []),
    "pf_transport_tdb_workspace_size": (C.c_size_t, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "pf_transport_tdb_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_int, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_size_t, C.c_void_p]),
    "pf_transport_tdb_mixed_workspace_size": (C.c_size_t, [C.c_int] * 6),
    "pf_transport_tdb_mixed_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_double, C.c_double, C.c_double, C.c_double,
                                             C.c_int, C.c_int,
                                             C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_size_t, C.c_void_p]),
    "pf_transport_tdb_mixed_ex_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_double, C.c_double, C.c_double, C.c_double,
                                                C.c_int, C.c_int, C.c_int,
                                                C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_size_t, C.c_void_p]),
    "pf_transport_tdb_mixed": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                         _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                         C.c_int, _dp, _ip, _ip,
                                         C.c_double, C.c_double, C.c_double, C.c_double,
                                         C.c_int, C.c_int,
                                         _dp, _ip, _ip]),
    "pf_transport_tdb_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_double, C.c_double, C.c_double, C.c_double,
                                           C.c_int, C.c_int,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p]),
    "pf_dyn_last_error": (C.c_char_p, []),
    "pf_gen_dyn_qe_tdb": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp,
                                    _dp, C.c_int, _dp, _ip, _dp, _dp, _dp, C.c_int, C.c_int,
                                    C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "pf_cond_last_error": (C.c_char_p, []),
    "pf_landauer_conductance": (C.c_int, [C.c_int, _dp, _dp, C.c_int, _dp, C.c_double, _dp]),
    "pf_grad_last_error": (C.c_char_p, []),
    "pf_transport_tdb_grad_workspace_size": (C.c_size_t, [C.c_int] * 8),
    "pf_transport_tdb_grad_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                            C.c_int, C.c_int,
                                            C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_size_t, C.c_void_p]),
    "pf_modes_last_error": (C.c_char_p, []),
    "pf_mixed_stage_timing": (C.c_int, [C.c_int]),
    "pf_tiled_set_tuning": (C.c_int, [C.c_int, C.c_int]),
    "pf_tiled_layout": (C.c_int, [C.c_int] * 5 + [C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "pf_mixed_stage_times": (C.c_int, [C.POINTER(C.c_float), C.c_int]),
    "pf_transport_tdb_blocks_workspace_size": (C.c_size_t, [C.c_int] * 5),
    "pf_transport_tdb_blocks_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                              C.c_void_p, C.c_void_p, C.c_void_p]
                                    + [C.c_void_p] * 10 + [C.c_void_p, C.c_size_t, C.c_void_p]),
    "pf_transport_tdb_modes_workspace_size": (C.c_size_t, [C.c_int] * 5),
    "pf_transport_tdb_modes_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                             C.c_double, C.c_double, C.c_double,
                                             C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int,
                                             C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_size_t, C.c_void_p]),
    "pf_transport_tdb_modes_ex_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                                C.c_double, C.c_double, C.c_double,
                                                C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int,
                                                C.c_void_p, C.c_int,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_size_t, C.c_void_p]),
    "pf_transport_tdb_modes_md2md_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                   C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                   C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                                   C.c_double, C.c_double, C.c_double,
                                                   C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int,
                                                   C.c_void_p, C.c_int,
                                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                   C.c_void_p, C.c_size_t, C.c_void_p]),
    "pf_transport_tdb_modes_permode_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                     C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                     C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                                     C.c_double, C.c_double, C.c_double,
                                                     C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int,
                                                     C.c_void_p,
                                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                     C.c_void_p, C.c_void_p, C.c_void_p,
                                                     C.c_void_p, C.c_size_t, C.c_void_p]),
    "pf_tiled_last_error": (C.c_char_p, []),
    "pf_transport_tdb_tiled_workspace_size": (C.c_size_t, [C.c_int] * 7),
    "pf_transport_tdb_tiled_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                             C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_size_t, C.c_void_p]),
    "pf_transport_tdb_tiled_circ_workspace_size": (C.c_size_t, [C.c_int] * 9),
    "pf_transport_tdb_tiled_circ_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                  C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                  C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                                  C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double),
                                                  C.c_void_p, C.c_void_p, C.c_void_p,
                                                  C.c_void_p, C.c_size_t, C.c_void_p]),
    "pf_transport_tdb_tiled_ex_workspace_size": (C.c_size_t, [C.c_int] * 9),
    "pf_transport_tdb_tiled_ex_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                                C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double),
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_size_t, C.c_void_p]),
    "pf_tc_last_error": (C.c_char_p, []),
    "pf_tc_zgemm_workspace_size": (C.c_size_t, [C.c_int] * 6),
    "pf_tc_zgemm_dev": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                  C.c_void_p, C.c_int, C.c_longlong, C.c_void_p, C.c_int, C.c_longlong,
                                  C.c_double, C.c_void_p, C.c_int, C.c_longlong, C.c_int,
                                  C.c_void_p, C.c_size_t, C.c_void_p]),
    "pf_fullh_last_error": (C.c_char_p, []),
    "pf_gen_dyn": (C.c_int, [C.c_int] * 7 + [_dp, _ip, C.c_int, _ip, _dp, _dp, _dp, C.c_int, _dp, C.c_int, _dp]),
    "pf_gen_dyn_dev": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_int] + [C.c_void_p] * 7
                       + [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "pf_dense_to_tdb_dev": (C.c_int, [C.c_int, C.c_int, C.c_void_p] + [C.c_int] * 5 + [C.c_void_p, C.c_int]
                            + [C.c_void_p] * 10),
    "pf_buttiker_last_error": (C.c_char_p, []),
    "pf_buttiker_tdb": (C.c_int, [C.c_int] * 5 + [_dp] * 8 + [C.c_int, _dp, _ip, _ip] + [_dp] * 6
                        + [C.c_double] * 4 + [C.c_int] + [_dp] * 7 + [_ip]),
    "pf_tb_last_error": (C.c_char_p, []),
    "pf_tb_hk_blocks": (C.c_int, [C.c_int, _dp, _ip, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, _dp, C.c_double,
                                  C.c_int, _dp, C.c_int, _ip, _dp]),
    "pf_transport_tdb": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                   _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                   C.c_int, _dp, _ip, _ip,
                                   C.c_double, C.c_double, C.c_double, C.c_double,
                                   C.c_int, C.c_int,
                                   _dp, _dp, _ip, _ip]),
}


class PFError(RuntimeError):
    """Error reported by the C ABI (message from pf_last_error)."""

    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def lib_path():
    return LIB


def load():
    """Load (once) and return the ctypes library handle."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        raise ImportError(
            f"{LIB} is missing: build it with `python -m phinfortran_gb300.build` "
            "(the engine has no CPU fallback)")
    lib = C.CDLL(LIB)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc):
    if rc != 0:
        msg = load().pf_last_error().decode(errors="replace")
        raise PFError(rc, msg)
    return rc
