"""Restatement of the primitive-cell unfolding of a lead mode (oracle;
tests only): find_k_pc (negf/dyn.f90:770-889) with compare_evs
(:662-768), group_velocity_pc_qe (:595-659), gen_dyn_pc_qe_k
(:2537-2635), in_ws and find_min_dist (negf/util.f90:589-638, 969-984) and
the primitive-cell set-up of read_input (negf/input.f90:587-711).

For a propagating mode with unfolded wavevector k (velocity_mat.f90:
2353-2360) the reference looks for the primitive-cell wavevector that
carries the same frequency: if k sits on the boundary of the unit cell's
Brillouin zone it is kept, otherwise every k + G (G a unit-cell reciprocal
vector, |components| <= max(n_bloch_x, n_bloch_y)) inside the primitive
Brillouin zone is tried, and a candidate counts when a primitive-cell
band lies within 1e-2 of sqrt(E).  The per-k files then carry the
candidate of smallest |k| and the group velocity of the first one.
"""
from __future__ import annotations

import numpy as np

PI = 3.141592653589793238   # negf/util.f90:5


def rotate_z(v, ang):
    """negf/util.f90:901-919 (rows are vectors)."""
    c, s = np.cos(ang), np.sin(ang)
    out = np.array(v, dtype=np.float64, copy=True)
    out[:, 0] = v[:, 0] * c - v[:, 1] * s
    out[:, 1] = v[:, 0] * s + v[:, 1] * c
    return out


def primitive_cell(latvec, scaled, species, lscale, mass_no):
    """negf/input.f90:587-711: lattice vectors scaled and turned by pi/4
    about z, atoms from scaled coordinates, the primitive-cell atoms those
    with crystal coordinates in (-0.001, 0.999); recivec_pc = 2 pi
    inv(latvec)^T.  Returns (positions_pc, recivec_pc, mass_uc)."""
    lat = rotate_z(np.asarray(latvec, dtype=np.float64) * lscale, PI / 4.0)
    pos_uc = np.asarray(scaled, dtype=np.float64) @ lat
    mass_uc = np.asarray(mass_no, dtype=np.float64)[np.asarray(species) - 1]
    rec = np.linalg.inv(lat)
    crys = pos_uc @ rec
    keep = np.all((crys < 0.999) & (crys > -0.001), axis=1)
    return pos_uc[keep], 2 * PI * rec.T, mass_uc


class PcDyn:
    """gen_dyn_pc_qe_k with its k-independent part precomputed: the terms
    (i, j, a, b, c) of the QE force constants that survive the
    Wigner-Seitz weighting, as weights, 3x3 blocks and bond vectors."""

    def __init__(self, qe, natoms_pc, mass_uc):
        pos, cell, fc = qe["pos"], qe["cell"], qe["fc"]
        rws, rd = qe["rws"], qe["rd"]
        nx, ny, nz = qe["nxyz"] if "nxyz" in qe else (qe["nx"], qe["ny"], qe["nz"])
        natm = pos.shape[0]
        ivcell = np.linalg.inv(cell)
        self.npc = natoms_pc
        shifts = np.array([(a, b, c) for a in range(-2 * nx, 2 * nx + 1) for b in range(-2 * ny, 2 * ny + 1)
                           for c in range(-2 * nz, 2 * nz + 1)], dtype=np.float64)
        rows, cols, blocks, drs = [], [], [], []
        for i in range(natoms_pc):
            for j in range(natm):
                dr = -(shifts @ cell) + pos[j] - pos[i]
                ixyz = (dr - (pos[j] - pos[i])) @ ivcell
                df = dr @ rws.T - rd[None, :]
                out = (df > 1.0e-5).any(axis=1)
                nreq = 1 + (np.abs(df) <= 1.0e-5).sum(axis=1)
                for t in np.nonzero(~out)[0]:
                    aa, bb, cc = (-int(np.sign(x) * np.floor(abs(x) + 0.5)) for x in ixyz[t])   # -idnint
                    w = 1.0 / nreq[t]
                    blk = w * fc[:, :, i, j, aa % nx, bb % ny, cc % nz] / np.sqrt(mass_uc[i] * mass_uc[j])
                    rows.append(i)
                    cols.append(j % natoms_pc)
                    blocks.append(blk)
                    drs.append(dr[t])
        rows, cols = np.array(rows), np.array(cols)
        blocks, drs = np.array(blocks), np.array(drs)
        # grouped by the (i, j mod natoms_pc) block they add to, in term order
        self.groups = []
        for i in range(natoms_pc):
            for j in range(natoms_pc):
                sel = np.nonzero((rows == i) & (cols == j))[0]
                self.groups.append((i, j, blocks[sel], drs[sel]))

    def __call__(self, k):
        n = 3 * self.npc
        k = np.asarray(k, dtype=np.float64)
        dyn = np.zeros((n, n), dtype=np.complex128)
        for i, j, blk, dr in self.groups:
            ph = np.exp(1j * (dr @ k))
            dyn[3 * i:3 * i + 3, 3 * j:3 * j + 3] = np.einsum("t,tmn->mn", ph, blk)
        return 0.5 * (dyn + dyn.conj().T)


def group_velocity(dynk, k, devi=1.0e-5):
    """group_velocity_pc_qe: eigenvalues (ascending) and the velocity of
    every band from central differences of D(k) (step 1e-5)."""
    k = np.asarray(k, dtype=np.float64)
    eigs, evs = np.linalg.eigh(dynk(k))
    vels = np.zeros((eigs.size, 3))
    for i in range(3):
        km, kp = k.copy(), k.copy()
        km[i] -= devi
        kp[i] += devi
        dh = (dynk(kp) - dynk(km)) / (2.0 * devi)
        vm = evs.conj().T @ dh @ evs
        vels[:, i] = np.real(np.diag(vm)) / (2 * np.sqrt(np.abs(eigs)))
    return eigs, vels


_M125 = np.array([(i1, i2, i3) for i1 in range(-2, 3) for i2 in range(-2, 3) for i3 in range(-2, 3)], float)


def in_ws_many(a, ks):
    """negf/util.f90:589-638 for every row of ks: 2 on a zone boundary
    (the two smallest distances to lattice points agree within 1e-5),
    1 inside (the origin is the nearest), 0 outside."""
    d = ks[:, None, :] - (_M125 @ a)[None, :, :]
    dist = np.einsum("kij,kij->ki", d, d)
    imin = np.argmin(dist, axis=1)
    dmin = dist[np.arange(ks.shape[0]), imin]
    rest = dist.copy()
    rest[np.arange(ks.shape[0]), imin] = np.inf
    dmin2 = rest.min(axis=1)
    out = np.zeros(ks.shape[0], dtype=np.int64)
    out[np.abs(dist[:, 62] - dmin) < 1.0e-5] = 1
    out[np.abs(dmin2 - dmin) < 1.0e-5] = 2
    return out


def in_ws(a, k):
    return int(in_ws_many(a, np.asarray(k, dtype=np.float64)[None, :])[0])


def find_k_pc(E, k_uc, reci_uc, recivec_pc, dynk, l):
    """(k_pc, v_pc) of one mode as the per-k files carry them: the candidate
    of smallest |k| (zero when there is none) and the velocity of the
    first candidate (zero when none matched)."""
    k_uc = np.asarray(k_uc, dtype=np.float64)
    w = np.sqrt(E)
    kpc, vpc = [], []
    if in_ws(reci_uc, k_uc) == 2:
        kpc.append(k_uc)
        eigs, vels = group_velocity(dynk, k_uc)
        v = np.zeros(3)
        for i in range(eigs.size):
            if abs(w - np.sqrt(abs(eigs[i]))) < 1.0e-2:
                v = vels[i]
        vpc.append(v)
    else:
        g = np.array([(i1, i2, i3) for i1 in range(-l, l + 1) for i2 in range(-l, l + 1)
                      for i3 in range(-l, l + 1)], float)
        cand = k_uc[None, :] + g @ reci_uc
        inside = in_ws_many(recivec_pc, cand)
        for kp in cand[inside != 0]:
            eigs, vels = group_velocity(dynk, kp)
            hit = None
            for i in range(eigs.size):
                if abs(w - np.sqrt(abs(eigs[i]))) < 1.0e-2:
                    hit = vels[i]
            if hit is not None:
                kpc.append(kp)
                vpc.append(hit)
    if not kpc:
        return np.zeros(3), np.zeros(3)
    kabs = [np.sqrt(x @ x) for x in kpc]
    return kpc[int(np.argmin(kabs))], vpc[0]
