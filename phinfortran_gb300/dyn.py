"""Host mirror of gen_dyn_qe_tdb (negf/dyn.f90:1436-1480) over the C ABI.

``gen_dyn_qe_tdb`` takes the arrays the phonon driver holds after read_qe_fc
(negf/fc.f90:103-325) and returns the tdb block set of every requested
transverse q, assembled on the GPU by pf_gen_dyn_qe_tdb.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi

_FAMILIES = ("HL", "HLv", "HR", "HRv", "Hd", "Hdv", "Hld", "Hrd")


def _f64(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def _ptr(a, ctype=C.c_double):
    return a.ctypes.data_as(C.POINTER(ctype))


def gen_dyn_qe_tdb(kgrid, *, fc, cell, pos, cell_all, pos_all, idxall, mass_all, rws, rd,
                   n_bloch_x, n_bloch_y, buffer_left, period_left, buffer_right, period_right,
                   nlayer, natm_layer):
    """Blocks for every row of ``kgrid`` (nq x 3 fractional).

    ``fc`` is fc_qe(3,3,nat,nat,nx,ny,nz); ``cell``/``cell_all`` have one
    lattice vector per row; ``idxall`` is 0-based (converted to the
    reference's 1-based convention here).  Returns a dict of arrays with a
    leading q axis: HL (nq, 3pl, 3pl), ..., Hd (nq, nlayer, 3na, 3na).
    """
    lib = _abi.load()
    kg = np.atleast_2d(np.asarray(kgrid, dtype=np.float64))
    nq = kg.shape[0]
    fc = _f64(fc)
    nat, nx, ny, nz = fc.shape[2], fc.shape[4], fc.shape[5], fc.shape[6]
    natall = pos_all.shape[0]
    idx1 = np.ascontiguousarray(np.asarray(idxall) + 1, dtype=np.int32)
    pl, pr, na = 3 * period_left, 3 * period_right, 3 * natm_layer
    shapes = dict(HL=(pl, pl), HLv=(pl, pl), HR=(pr, pr), HRv=(pr, pr), Hd=(nlayer, na, na),
                  Hdv=(max(nlayer - 1, 0), na, na), Hld=(pl, na), Hrd=(pr, na))
    # interleaved complex buffers, column-major within each block
    raw = {k: np.zeros(2 * nq * int(np.prod(s)), np.float64) for k, s in shapes.items()}
    rc = lib.pf_gen_dyn_qe_tdb(nat, nx, ny, nz, _ptr(fc), _ptr(_f64(cell)), _ptr(_f64(cell_all)),
                               _ptr(_f64(pos)), natall, _ptr(_f64(pos_all)), _ptr(idx1, C.c_int),
                               _ptr(_f64(mass_all)), _ptr(_f64(rws)), _ptr(_f64(rd)), n_bloch_x, n_bloch_y,
                               buffer_left, period_left, buffer_right, period_right, nlayer, natm_layer, nq,
                               _ptr(_f64(kg)), *[_ptr(raw[k]) for k in _FAMILIES])
    if rc != 0:
        raise _abi.PFError(rc, lib.pf_dyn_last_error().decode(errors="replace"))
    out = {}
    for k, s in shapes.items():
        z = raw[k].view(np.complex128)
        if len(s) == 2:
            out[k] = z.reshape((nq, s[1], s[0])).swapaxes(-1, -2)
        else:
            out[k] = z.reshape((nq, s[0], s[2], s[1])).swapaxes(-1, -2)
    return out
