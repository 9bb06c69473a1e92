"""Tight-binding H(k) of tb/hamiltonian.f90 (oracle; tests only).

Restates gen_ham (tb/hamiltonian.f90:444-519) and the Slater-Koster
two-centre table V_sk (tb/hamiltonian.f90:74-417) with its power-law
scaling V_term (tb/hamiltonian.f90:28-55) and onsite rule (:57-72):

* element (i, j) = sum over the 27 cell images (i1, i2, i3 in -1..1) with
  |r_ij| < r_cutoff of exp(i r_ij . k_cart) V_ij, where V_ij is the onsite
  value when the two orbitals sit on the same atom -- for every image of it,
  not only the zero shift -- and V_sk otherwise;
* V_term = V(si, sj, n1, n2, type) (d0 / |r| / ang)^Vn(si, sj, n1, n2, type),
  d0 = r_d(si, sj), ang = 1e-10;
* the reversed pairs ("pxs", "dxypx", ...) use the species-swapped V with
  the table's own signs, and "dz2dz2" uses the swapped V as well;
* sqrt(3.0) is a single-precision Fortran literal (1.7320508 as float32);
* H = 0.5 (H + H^H) at the end (tb/util.f90:709-718).

Orbital codes: 0 s, 1 px, 2 py, 3 pz, 4 dxy, 5 dyz, 6 dxz, 7 dx2-y2, 8 dz2,
9 s*; principal numbers (get_principal_number): s 1, p 2, d 3, s* 4.
V, Vn: (nspecies, nspecies, 4, 4, 4) indexed [si, sj, n1-1, n2-1, type-1]
with type 1 onsite, 2 sigma, 3 pi, 4 delta.
"""
from __future__ import annotations

import numpy as np

ANG = 1.0e-10
S3 = float(np.float32(np.sqrt(np.float32(3.0))))   # Fortran sqrt(3.0), real(4)
PRINCIPAL = [1, 2, 2, 2, 3, 3, 3, 3, 3, 4]
NAMES = ["s", "px", "py", "pz", "dxy", "dyz", "dxz", "dx2-y2", "dz2", "s*"]


def v_term(V, Vn, r_d, i, j, n1, n2, vt, dist):
    d0 = r_d[i, j]
    npow = Vn[i, j, n1 - 1, n2 - 1, vt - 1]
    return V[i, j, n1 - 1, n2 - 1, vt - 1] * (d0 / dist / ANG) ** npow


def onsite(V, i, j, o1, o2):
    if o1 == o2:
        n = PRINCIPAL[o1]
        return V[i, j, n - 1, n - 1, 0]
    return 0.0


def v_sk(V, Vn, r_d, i, j, o1, o2, r):
    """Slater-Koster element between orbital o1 of species i and o2 of
    species j for the bond vector r (tb/hamiltonian.f90:74-417)."""
    dist = np.sqrt(r[0] ** 2 + r[1] ** 2 + r[2] ** 2)
    l, m, n = r[0] / dist, r[1] / dist, r[2] / dist
    T = lambda a, b, n1, n2, vt: v_term(V, Vn, r_d, a, b, n1, n2, vt, dist)
    key = NAMES[o1] + NAMES[o2]
    l2, m2, n2_ = l * l, m * m, n * n
    c = {
        "ss": lambda: T(i, j, 1, 1, 2),
        "spx": lambda: l * T(i, j, 1, 2, 2), "pxs": lambda: -l * T(j, i, 1, 2, 2),
        "spy": lambda: m * T(i, j, 1, 2, 2), "pys": lambda: -m * T(j, i, 1, 2, 2),
        "spz": lambda: n * T(i, j, 1, 2, 2), "pzs": lambda: -n * T(j, i, 1, 2, 2),
        "pxpx": lambda: l2 * T(i, j, 2, 2, 2) + (1 - l2) * T(i, j, 2, 2, 3),
        "pypy": lambda: m2 * T(i, j, 2, 2, 2) + (1 - m2) * T(i, j, 2, 2, 3),
        "pzpz": lambda: n2_ * T(i, j, 2, 2, 2) + (1 - n2_) * T(i, j, 2, 2, 3),
        "pxpy": lambda: l * m * T(i, j, 2, 2, 2) - l * m * T(i, j, 2, 2, 3),
        "pypx": lambda: l * m * T(i, j, 2, 2, 2) - l * m * T(i, j, 2, 2, 3),
        "pypz": lambda: m * n * T(i, j, 2, 2, 2) - m * n * T(i, j, 2, 2, 3),
        "pzpy": lambda: m * n * T(i, j, 2, 2, 2) - m * n * T(i, j, 2, 2, 3),
        "pxpz": lambda: l * n * T(i, j, 2, 2, 2) - l * n * T(i, j, 2, 2, 3),
        "pzpx": lambda: l * n * T(i, j, 2, 2, 2) - l * n * T(i, j, 2, 2, 3),
        "sdxy": lambda: S3 * (l * m) * T(i, j, 1, 3, 2), "dxys": lambda: S3 * (l * m) * T(j, i, 1, 3, 2),
        "sdyz": lambda: S3 * (m * n) * T(i, j, 1, 3, 2), "dyzs": lambda: S3 * (m * n) * T(j, i, 1, 3, 2),
        "sdxz": lambda: S3 * (l * n) * T(i, j, 1, 3, 2), "dxzs": lambda: S3 * (l * n) * T(j, i, 1, 3, 2),
        "sdx2-y2": lambda: (S3 / 2) * (l2 - m2) * T(i, j, 1, 3, 2),
        "dx2-y2s": lambda: (S3 / 2) * (l2 - m2) * T(j, i, 1, 3, 2),
        "sdz2": lambda: (n2_ - (l2 + m2) / 2) * T(i, j, 1, 3, 2),
        "dz2s": lambda: (n2_ - (l2 + m2) / 2) * T(j, i, 1, 3, 2),
        "pxdxy": lambda: S3 * (l2 * m) * T(i, j, 2, 3, 2) + m * (1 - 2 * l2) * T(i, j, 2, 3, 3),
        "dxypx": lambda: -S3 * (l2 * m) * T(j, i, 2, 3, 2) - m * (1 - 2 * l2) * T(j, i, 2, 3, 3),
        "pxdyz": lambda: S3 * (l * m * n) * T(i, j, 2, 3, 2) - 2 * (l * m * n) * T(i, j, 2, 3, 3),
        "dyzpx": lambda: -S3 * (l * m * n) * T(j, i, 2, 3, 2) + 2 * (l * m * n) * T(j, i, 2, 3, 3),
        "pxdxz": lambda: S3 * (l2 * n) * T(i, j, 2, 3, 2) + n * (1 - 2 * l2) * T(i, j, 2, 3, 3),
        "dxzpx": lambda: -S3 * (l2 * n) * T(j, i, 2, 3, 2) - n * (1 - 2 * l2) * T(j, i, 2, 3, 3),
        "pydxy": lambda: S3 * (m2 * l) * T(i, j, 2, 3, 2) + l * (1 - 2 * m2) * T(i, j, 2, 3, 3),
        "dxypy": lambda: -S3 * (m2 * l) * T(j, i, 2, 3, 2) - l * (1 - 2 * m2) * T(j, i, 2, 3, 3),
        "pydyz": lambda: S3 * (m2 * n) * T(i, j, 2, 3, 2) + n * (1 - 2 * m2) * T(i, j, 2, 3, 3),
        "dyzpy": lambda: -S3 * (m2 * n) * T(j, i, 2, 3, 2) - n * (1 - 2 * m2) * T(j, i, 2, 3, 3),
        "pydxz": lambda: S3 * (l * m * n) * T(i, j, 2, 3, 2) - 2 * (l * m * n) * T(i, j, 2, 3, 3),
        "dxzpy": lambda: -S3 * (l * m * n) * T(j, i, 2, 3, 2) + 2 * (l * m * n) * T(j, i, 2, 3, 3),
        "pzdxy": lambda: S3 * (l * m * n) * T(i, j, 2, 3, 2) - 2 * (l * m * n) * T(i, j, 2, 3, 3),
        "dxypz": lambda: -S3 * (l * m * n) * T(j, i, 2, 3, 2) + 2 * (l * m * n) * T(j, i, 2, 3, 3),
        "pzdyz": lambda: S3 * (n2_ * m) * T(i, j, 2, 3, 2) + m * (1 - 2 * n2_) * T(i, j, 2, 3, 3),
        "dyzpz": lambda: -S3 * (n2_ * m) * T(j, i, 2, 3, 2) - m * (1 - 2 * n2_) * T(j, i, 2, 3, 3),
        "pzdxz": lambda: S3 * (n2_ * l) * T(i, j, 2, 3, 2) + l * (1 - 2 * n2_) * T(i, j, 2, 3, 3),
        "dxzpz": lambda: -S3 * (n2_ * l) * T(j, i, 2, 3, 2) - l * (1 - 2 * n2_) * T(j, i, 2, 3, 3),
        "pxdx2-y2": lambda: (S3 / 2) * l * (l2 - m2) * T(i, j, 2, 3, 2) + l * (1 - l2 + m2) * T(i, j, 2, 3, 3),
        "dx2-y2px": lambda: -(S3 / 2) * l * (l2 - m2) * T(j, i, 2, 3, 2) - l * (1 - l2 + m2) * T(j, i, 2, 3, 3),
        "pydx2-y2": lambda: (S3 / 2) * m * (l2 - m2) * T(i, j, 2, 3, 2) - m * (1 + l2 - m2) * T(i, j, 2, 3, 3),
        "dx2-y2py": lambda: -(S3 / 2) * m * (l2 - m2) * T(j, i, 2, 3, 2) + m * (1 + l2 - m2) * T(j, i, 2, 3, 3),
        "pzdx2-y2": lambda: (S3 / 2) * n * (l2 - m2) * T(i, j, 2, 3, 2) - n * (l2 - m2) * T(i, j, 2, 3, 3),
        "dx2-y2pz": lambda: -(S3 / 2) * n * (l2 - m2) * T(j, i, 2, 3, 2) + n * (l2 - m2) * T(j, i, 2, 3, 3),
        "pxdz2": lambda: l * (n2_ - (l2 + m2) / 2) * T(i, j, 2, 3, 2) - S3 * l * n2_ * T(i, j, 2, 3, 3),
        "dz2px": lambda: -l * (n2_ - (l2 + m2) / 2) * T(j, i, 2, 3, 2) + S3 * l * n2_ * T(j, i, 2, 3, 3),
        "pydz2": lambda: m * (n2_ - (l2 + m2) / 2) * T(i, j, 2, 3, 2) - S3 * m * n2_ * T(i, j, 2, 3, 3),
        "dz2py": lambda: -m * (n2_ - (l2 + m2) / 2) * T(j, i, 2, 3, 2) + S3 * m * n2_ * T(j, i, 2, 3, 3),
        "pzdz2": lambda: n * (n2_ - (l2 + m2) / 2) * T(i, j, 2, 3, 2) + S3 * n * (l2 + m2) * T(i, j, 2, 3, 3),
        "dz2pz": lambda: -n * (n2_ - (l2 + m2) / 2) * T(j, i, 2, 3, 2) - S3 * n * (l2 + m2) * T(j, i, 2, 3, 3),
        "dxydxy": lambda: (3 * l2 * m2 * T(i, j, 3, 3, 2) + (l2 + m2 - 4 * l2 * m2) * T(i, j, 3, 3, 3)
                           + (n2_ + l2 * m2) * T(i, j, 3, 3, 4)),
        "dyzdyz": lambda: (3 * m2 * n2_ * T(i, j, 3, 3, 2) + (m2 + n2_ - 4 * m2 * n2_) * T(i, j, 3, 3, 3)
                           + (l2 + m2 * n2_) * T(i, j, 3, 3, 4)),
        "dxzdxz": lambda: (3 * l2 * n2_ * T(i, j, 3, 3, 2) + (l2 + n2_ - 4 * l2 * n2_) * T(i, j, 3, 3, 3)
                           + (m2 + l2 * n2_) * T(i, j, 3, 3, 4)),
        "dxydyz": lambda: (3 * l * m2 * n * T(i, j, 3, 3, 2) + l * n * (1 - 4 * m2) * T(i, j, 3, 3, 3)
                           + l * n * (m2 - 1) * T(i, j, 3, 3, 4)),
        "dyzdxy": lambda: (3 * l * m2 * n * T(j, i, 3, 3, 2) + l * n * (1 - 4 * m2) * T(j, i, 3, 3, 3)
                           + l * n * (m2 - 1) * T(j, i, 3, 3, 4)),
        "dxydxz": lambda: (3 * m * l2 * n * T(i, j, 3, 3, 2) + m * n * (1 - 4 * l2) * T(i, j, 3, 3, 3)
                           + m * n * (l2 - 1) * T(i, j, 3, 3, 4)),
        "dxzdxy": lambda: (3 * m * l2 * n * T(j, i, 3, 3, 2) + m * n * (1 - 4 * l2) * T(j, i, 3, 3, 3)
                           + m * n * (l2 - 1) * T(j, i, 3, 3, 4)),
        "dyzdxz": lambda: (3 * m * n2_ * l * T(i, j, 3, 3, 2) + m * l * (1 - 4 * n2_) * T(i, j, 3, 3, 3)
                           + m * l * (n2_ - 1) * T(i, j, 3, 3, 4)),
        "dxzdyz": lambda: (3 * m * n2_ * l * T(j, i, 3, 3, 2) + m * l * (1 - 4 * n2_) * T(j, i, 3, 3, 3)
                           + m * l * (n2_ - 1) * T(j, i, 3, 3, 4)),
        "dxydx2-y2": lambda: ((3.0 / 2) * l * m * (l2 - m2) * T(i, j, 3, 3, 2) + 2 * l * m * (m2 - l2) * T(i, j, 3, 3, 3)
                              + (1.0 / 2) * l * m * (l2 - m2) * T(i, j, 3, 3, 4)),
        "dx2-y2dxy": lambda: ((3.0 / 2) * l * m * (l2 - m2) * T(j, i, 3, 3, 2) + 2 * l * m * (m2 - l2) * T(j, i, 3, 3, 3)
                              + (1.0 / 2) * l * m * (l2 - m2) * T(j, i, 3, 3, 4)),
        "dyzdx2-y2": lambda: ((3.0 / 2) * m * n * (l2 - m2) * T(i, j, 3, 3, 2)
                              - m * n * (1 + 2 * (l2 - m2)) * T(i, j, 3, 3, 3)
                              + m * n * (1 + (l2 - m2) / 2) * T(i, j, 3, 3, 4)),
        "dx2-y2dyz": lambda: ((3.0 / 2) * m * n * (l2 - m2) * T(j, i, 3, 3, 2)
                              - m * n * (1 + 2 * (l2 - m2)) * T(j, i, 3, 3, 3)
                              + m * n * (1 + (l2 - m2) / 2) * T(j, i, 3, 3, 4)),
        "dxzdx2-y2": lambda: ((3.0 / 2) * l * n * (l2 - m2) * T(i, j, 3, 3, 2)
                              + l * n * (1 - 2 * (l2 - m2)) * T(i, j, 3, 3, 3)
                              - l * n * (1 - (l2 - m2) / 2) * T(i, j, 3, 3, 4)),
        "dx2-y2dxz": lambda: ((3.0 / 2) * l * n * (l2 - m2) * T(j, i, 3, 3, 2)
                              + l * n * (1 - 2 * (l2 - m2)) * T(j, i, 3, 3, 3)
                              - l * n * (1 - (l2 - m2) / 2) * T(j, i, 3, 3, 4)),
        "dxydz2": lambda: (S3 * l * m * (n2_ - (l2 + m2) / 2) * T(i, j, 3, 3, 2) - (2 * S3) * l * m * n2_ * T(i, j, 3, 3, 3)
                           + (S3 / 2) * l * m * (1 + n2_) * T(i, j, 3, 3, 4)),
        "dz2dxy": lambda: (S3 * l * m * (n2_ - (l2 + m2) / 2) * T(j, i, 3, 3, 2) - (2 * S3) * l * m * n2_ * T(j, i, 3, 3, 3)
                           + (S3 / 2) * l * m * (1 + n2_) * T(j, i, 3, 3, 4)),
        "dyzdz2": lambda: (S3 * m * n * (n2_ - (l2 + m2) / 2) * T(i, j, 3, 3, 2)
                           + S3 * m * n * (l2 + m2 - n2_) * T(i, j, 3, 3, 3)
                           - (S3 / 2) * m * n * (l2 + m2) * T(i, j, 3, 3, 4)),
        "dz2dyz": lambda: (S3 * m * n * (n2_ - (l2 + m2) / 2) * T(j, i, 3, 3, 2)
                           + S3 * m * n * (l2 + m2 - n2_) * T(j, i, 3, 3, 3)
                           - (S3 / 2) * m * n * (l2 + m2) * T(j, i, 3, 3, 4)),
        "dxzdz2": lambda: (S3 * l * n * (n2_ - (l2 + m2) / 2) * T(i, j, 3, 3, 2)
                           + S3 * l * n * (l2 + m2 - n2_) * T(i, j, 3, 3, 3)
                           - (S3 / 2) * l * n * (l2 + m2) * T(i, j, 3, 3, 4)),
        "dz2dxz": lambda: (S3 * l * n * (n2_ - (l2 + m2) / 2) * T(j, i, 3, 3, 2)
                           + S3 * l * n * (l2 + m2 - n2_) * T(j, i, 3, 3, 3)
                           - (S3 / 2) * l * n * (l2 + m2) * T(j, i, 3, 3, 4)),
        "dx2-y2dx2-y2": lambda: ((3.0 / 4) * ((l2 - m2) ** 2) * T(i, j, 3, 3, 2)
                                 + (l2 + m2 - (l2 - m2) ** 2) * T(i, j, 3, 3, 3)
                                 + (n2_ + ((l2 - m2) ** 2) / 4) * T(i, j, 3, 3, 4)),
        "dx2-y2dz2": lambda: ((S3 / 2) * (l2 - m2) * (n2_ - (l2 + m2) / 2) * T(i, j, 3, 3, 2)
                              + S3 * n2_ * (m2 - l2) * T(i, j, 3, 3, 3)
                              + (S3 / 4) * (1 + n2_) * (l2 - m2) * T(i, j, 3, 3, 4)),
        "dz2dx2-y2": lambda: ((S3 / 2) * (l2 - m2) * (n2_ - (l2 + m2) / 2) * T(j, i, 3, 3, 2)
                              + S3 * n2_ * (m2 - l2) * T(j, i, 3, 3, 3)
                              + (S3 / 4) * (1 + n2_) * (l2 - m2) * T(j, i, 3, 3, 4)),
        "dz2dz2": lambda: (((n2_ - (l2 + m2) / 2) ** 2) * T(j, i, 3, 3, 2) + 3 * n2_ * (l2 + m2) * T(j, i, 3, 3, 3)
                           + (3.0 / 4) * ((l2 + m2) ** 2) * T(j, i, 3, 3, 4)),
        "s*s*": lambda: T(i, j, 4, 4, 2),
        "ss*": lambda: T(i, j, 1, 4, 2), "s*s": lambda: T(j, i, 1, 4, 2),
        "s*px": lambda: l * T(i, j, 4, 2, 2), "pxs*": lambda: -l * T(j, i, 4, 2, 2),
        "s*py": lambda: m * T(i, j, 4, 2, 2), "pys*": lambda: -m * T(j, i, 4, 2, 2),
        "s*pz": lambda: n * T(i, j, 4, 2, 2), "pzs*": lambda: -n * T(j, i, 4, 2, 2),
        "s*dxy": lambda: S3 * (l * m) * T(i, j, 4, 3, 2), "dxys*": lambda: S3 * (l * m) * T(j, i, 4, 3, 2),
        "s*dyz": lambda: S3 * (m * n) * T(i, j, 4, 3, 2), "dyzs*": lambda: S3 * (m * n) * T(j, i, 4, 3, 2),
        "s*dxz": lambda: S3 * (l * n) * T(i, j, 4, 3, 2), "dxzs*": lambda: S3 * (l * n) * T(j, i, 4, 3, 2),
        "s*dx2-y2": lambda: (S3 / 2) * (l2 - m2) * T(i, j, 4, 3, 2),
        "dx2-y2s*": lambda: (S3 / 2) * (l2 - m2) * T(j, i, 4, 3, 2),
        "s*dz2": lambda: (n2_ - (l2 + m2) / 2) * T(i, j, 4, 3, 2),
        "dz2s*": lambda: (n2_ - (l2 + m2) / 2) * T(j, i, 4, 3, 2),
    }
    f = c.get(key)
    return 0.0 if f is None else f()


def orbital_list(species, orbs):
    """Per-orbital (atom, species, code) rows in gen_ham's order."""
    rows = []
    for a, s in enumerate(species):
        for o in orbs[s]:
            rows.append((a, s, o))
    return rows


def gen_ham_raw(pos, species, orbs, V, Vn, r_d, latvec, r_cutoff, kfrac, recivec, rows_i=None, rows_j=None):
    """Raw (not yet Hermitised) gen_ham elements for the orbital row lists
    rows_i x rows_j (default: all orbitals)."""
    rows = orbital_list(species, orbs)
    ri = rows if rows_i is None else rows_i
    rj = rows if rows_j is None else rows_j
    kc = np.asarray(kfrac, dtype=np.float64) @ recivec
    shifts = [np.array([i1, i2, i3], dtype=np.float64) @ latvec
              for i1 in (-1, 0, 1) for i2 in (-1, 0, 1) for i3 in (-1, 0, 1)]
    H = np.zeros((len(ri), len(rj)), np.complex128)
    for a, (ia, si, oi) in enumerate(ri):
        for b, (ja, sj, oj) in enumerate(rj):
            acc = 0.0 + 0.0j
            for sh in shifts:
                r = pos[ja] - pos[ia] + sh
                if np.sqrt(r[0] ** 2 + r[1] ** 2 + r[2] ** 2) < r_cutoff:
                    v = onsite(V, si, sj, oi, oj) if ia == ja else v_sk(V, Vn, r_d, si, sj, oi, oj, r)
                    acc += np.exp(1j * np.dot(r, kc)) * v
            H[a, b] = acc
    return H


def gen_ham(pos, species, orbs, V, Vn, r_d, latvec, r_cutoff, kfrac, recivec):
    """Dense Hermitised H(k) (tb/hamiltonian.f90:444-519)."""
    H = gen_ham_raw(pos, species, orbs, V, Vn, r_d, latvec, r_cutoff, kfrac, recivec)
    return 0.5 * (H + H.conj().T)
