"""Tight-binding H(k) blocks through pf_tb_hk_blocks.

The electron driver builds the dense H(k) of the whole structure with
gen_ham (tb/hamiltonian.f90:444-519) and cuts the lead and device blocks
out of it; ``tb_blocks`` builds those blocks directly on the GPU for a list
of layers (atom ranges) and k points.  ``tdb_from_layers`` maps a layer
stack [lead cell -1, lead cell 0, device 1..L, lead cell N+1, lead cell
N+2] onto the transport entries' block names.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi

CODES = {"s": 0, "px": 1, "py": 2, "pz": 3, "dxy": 4, "dyz": 5, "dxz": 6, "dx2-y2": 7, "dz2": 8, "s*": 9}
MAX_ORB = 10   # PF_TB_MAX_ORB


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def tb_blocks(pos, species, orbitals, V, Vn, r_d, latvec, r_cutoff, kfrac, blk_atom):
    """pos (natoms, 3), species (natoms,) 0-based, orbitals: list (per
    species) of orbital names or codes, V / Vn (ns, ns, 4, 4, 4), r_d
    (ns, ns), latvec rows, kfrac (nk, 3), blk_atom (nblk + 1,) atom
    boundaries.  Returns (diag, upper): lists over k of lists of blocks."""
    lib = _abi.load()
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    species = np.ascontiguousarray(species, dtype=np.int32)
    ns = len(orbitals)
    norb = np.array([len(o) for o in orbitals], dtype=np.int32)
    codes = np.zeros((ns, MAX_ORB), dtype=np.int32)
    for s, lst in enumerate(orbitals):
        for i, o in enumerate(lst):
            codes[s, i] = CODES[o] if isinstance(o, str) else int(o)
    V = np.ascontiguousarray(V, dtype=np.float64)
    Vn = np.ascontiguousarray(Vn, dtype=np.float64)
    r_d = np.ascontiguousarray(r_d, dtype=np.float64)
    latvec = np.ascontiguousarray(latvec, dtype=np.float64)
    recivec = np.ascontiguousarray(2 * np.pi * np.linalg.inv(latvec).T)
    kfrac = np.ascontiguousarray(np.atleast_2d(kfrac), dtype=np.float64)
    blk_atom = np.ascontiguousarray(blk_atom, dtype=np.int32)
    nblk = blk_atom.size - 1
    orb_first = np.concatenate([[0], np.cumsum(norb[species])])
    sizes = [int(orb_first[blk_atom[i + 1]] - orb_first[blk_atom[i]]) for i in range(nblk)]
    per_k = sum(s * s for s in sizes) + sum(sizes[i] * sizes[i + 1] for i in range(nblk - 1))
    out = np.zeros(2 * kfrac.shape[0] * per_k)
    rc = lib.pf_tb_hk_blocks(pos.shape[0], _p(pos), _p(species, C.c_int), ns, _p(norb, C.c_int),
                             _p(codes, C.c_int), _p(V), _p(Vn), _p(r_d), _p(latvec), _p(recivec), float(r_cutoff),
                             kfrac.shape[0], _p(kfrac), nblk, _p(blk_atom, C.c_int), _p(out))
    if rc != 0:
        raise _abi.PFError(rc, lib.pf_tb_last_error().decode(errors="replace"))
    z = out.view(np.complex128).reshape(kfrac.shape[0], per_k)
    diag, upper = [], []
    for k in range(kfrac.shape[0]):
        off = 0
        dk, uk = [], []
        for s in sizes:
            dk.append(z[k, off:off + s * s].reshape(s, s).T.copy())
            off += s * s
        for i in range(nblk - 1):
            a, b = sizes[i], sizes[i + 1]
            uk.append(z[k, off:off + a * b].reshape(b, a).T.copy())
            off += a * b
        diag.append(dk)
        upper.append(uk)
    return diag, upper


def tdb_from_layers(diag, upper):
    """Block set of one k from a layer stack [lead -1, lead 0, device 1..L,
    lead N+1, lead N+2]: HL = H_{-1,-1}, HLv = H_{-1,0}, Hld = H_{0,1},
    Hd_j = H_{j,j}, Hdv_j = H_{j,j+1}, Hrd = H_{N+1,N} = H_{N,N+1}^H,
    HR = H_{N+2,N+2}, HRv = H_{N+2,N+1} = H_{N+1,N+2}^H."""
    nl = len(diag)
    L = nl - 4
    return dict(HL=diag[0], HLv=upper[0], Hld=upper[1], Hd=np.array(diag[2:2 + L]),
                Hdv=np.array(upper[2:1 + L]) if L > 1 else np.zeros((0,) + diag[2].shape, np.complex128),
                Hrd=upper[1 + L].conj().T, HR=diag[nl - 1], HRv=upper[nl - 2].conj().T)
