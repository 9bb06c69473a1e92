"""Block dynamical-matrix assembly of the tdb branch (oracle; tests only).

Restates ``gen_dyn_qe_tdb_k`` (negf/dyn.f90:1482-2080).  For one transverse
q it fills the eight block families

    Haml, Hamlv, Hamr, Hamrv  (lead cells)      dyn.f90:1568-1798
    Hamd(L), Hamdv(L-1)       (device layers)   dyn.f90:1800-1936
    Hamld, Hamrd              (lead-device)     dyn.f90:1938-2078

Each element is sum_{a,b} w * fc(m,n,iat,jat,t1,t2,t3) * exp(i dr.q)/sqrt(mi mj)
over transverse images a in [-nscx,nscx], b in [-nscy,nscy] (c = 0 only),
with the Wigner-Seitz weight w = 1/nreq from the 124 planes (dyn.f90:1571-1586).
The result is NOT hermitised (unlike gen_dyn, dyn.f90:139).
"""
from __future__ import annotations

import numpy as np

from .qe import PI, ceil_div


def _block(kpoint, rows, cols, pos_all, idxall, mass_all, qe, cell_all, nscx, nscy):
    """One block family: rows/cols are 0-based atom index ranges."""
    pos_uc = qe["pos"]
    fc = qe["fc"]
    nx, ny, nz = qe["nx"], qe["ny"], qe["nz"]
    ivcell = np.linalg.inv(qe["cell"])
    rws, rd = qe["rws"], qe["rd"]
    ni, nj = len(rows), len(cols)
    out = np.zeros((3 * ni, 3 * nj), dtype=np.complex128)
    ab = np.array([(a, b, 0) for a in range(-nscx, nscx + 1)
                   for b in range(-nscy, nscy + 1)], dtype=np.float64)
    shifts = ab @ cell_all                                  # (nab, 3)
    for bi, i in enumerate(rows):
        pi_, piu, mi = pos_all[i], pos_uc[idxall[i]], mass_all[i]
        for bj, j in enumerate(cols):
            pj, pju, mj = pos_all[j], pos_uc[idxall[j]], mass_all[j]
            dr = -shifts + pj - pi_                         # (nab, 3)
            ixyz = (dr - (pju - piu)) @ ivcell
            df = dr @ rws.T - rd[None, :]                   # (nab, 124)
            outside = (df > 1.0e-5).any(axis=1)
            nreq = 1 + (np.abs(df) <= 1.0e-5).sum(axis=1)
            w = np.where(outside, 0.0, 1.0 / nreq)
            # Fortran idnint rounds half away from zero
            aa = -np.trunc(ixyz + np.copysign(0.5, ixyz)).astype(np.int64)
            t1 = np.mod(aa[:, 0], nx)
            t2 = np.mod(aa[:, 1], ny)
            t3 = np.mod(aa[:, 2], nz)
            phase = np.exp(1j * (dr @ kpoint)) / np.sqrt(mi * mj)
            acc = np.zeros((3, 3), dtype=np.complex128)
            for s in np.nonzero(w > 0.0)[0]:
                acc += w[s] * fc[:, :, idxall[i], idxall[j], t1[s], t2[s], t3[s]] * phase[s]
            out[3 * bi:3 * bi + 3, 3 * bj:3 * bj + 3] = acc
    return out


def gen_dyn_qe_tdb_k(kgrid, qe, cell_all, pos_all, idxall, mass_all,
                     n_bloch_x, n_bloch_y, nz, buffer_left, period_left,
                     buffer_right, period_right, nlayer, natm_layer):
    """All tdb blocks for fractional ``kgrid`` (3,), negf/dyn.f90:1482-2080.

    Atom ranges use the reference's 1-based bounds converted to 0-based.
    Returns dict HL, HLv, HR, HRv, Hd (L,n,n), Hdv (L-1,n,n), Hld, Hrd.
    """
    cell_reci = 2 * PI * np.linalg.inv(qe["cell"]).T
    kpoint = np.asarray(kgrid, dtype=np.float64) @ cell_reci
    nscx = ceil_div(qe["nx"], n_bloch_x)
    nscy = ceil_div(qe["ny"], n_bloch_y)
    nat_all = pos_all.shape[0]
    args = (pos_all, idxall, mass_all, qe, cell_all, nscx, nscy)

    def rng(lo, hi):               # Fortran lo..hi inclusive, 1-based
        return list(range(lo - 1, hi))

    bl, pl, br, pr = buffer_left, period_left, buffer_right, period_right
    HL = _block(kpoint, rng(bl + 1, bl + pl), rng(bl + 1, bl + pl), *args)
    HLv = _block(kpoint, rng(bl + 1, bl + pl), rng(bl + pl + 1, bl + 2 * pl), *args)
    HR = _block(kpoint, rng(nat_all - br - pr + 1, nat_all - br),
                rng(nat_all - br - pr + 1, nat_all - br), *args)
    HRv = _block(kpoint, rng(nat_all - br - pr + 1, nat_all - br),
                 rng(nat_all - br - 2 * pr + 1, nat_all - br - pr), *args)
    ds = bl + 2 * pl
    Hd, Hdv = [], []
    for ilay in range(1, nlayer + 1):
        lay = rng(ds + (ilay - 1) * natm_layer + 1, ds + ilay * natm_layer)
        Hd.append(_block(kpoint, lay, lay, *args))
        if ilay < nlayer:
            nxt = rng(ds + ilay * natm_layer + 1, ds + (ilay + 1) * natm_layer)
            Hdv.append(_block(kpoint, lay, nxt, *args))
    Hld = _block(kpoint, rng(bl + pl + 1, bl + 2 * pl), rng(ds + 1, ds + natm_layer), *args)
    Hrd = _block(kpoint, rng(nat_all - br - 2 * pr + 1, nat_all - br - pr),
                 rng(ds + (nlayer - 1) * natm_layer + 1, ds + nlayer * natm_layer), *args)
    n = 3 * natm_layer
    return dict(HL=HL, HLv=HLv, HR=HR, HRv=HRv,
                Hd=np.array(Hd), Hdv=np.array(Hdv) if Hdv else np.zeros((0, n, n), complex),
                Hld=Hld, Hrd=Hrd)
