"""Primitive-cell wavevector and group velocity of lead modes, for the
primitive-cell columns of the per-k mode files.

The reference calls find_k_pc (negf/dyn.f90:770-889) for every
propagating mode of the four lead problems (velocity_mat.f90:2370-2383)
and writes, for each incoming mode, the primitive-cell k of smallest norm
among the candidates k + G that carry a band within 1e-2 of sqrt(E), and
the group velocity of the first candidate (write_data.f90:3-176).  The
candidates are the unit-cell reciprocal translates k + G, |G components|
<= max(n_bloch_x, n_bloch_y), inside the primitive Brillouin zone
(in_ws, negf/util.f90:589-638), or k itself when it lies on the unit
cell's zone boundary.  The bands come from the primitive-cell dynamical
matrix built from the QE force constants with Wigner-Seitz weights
(gen_dyn_pc_qe_k, negf/dyn.f90:2537-2635) and the velocities from central
differences of it (group_velocity_pc_qe, :595-659).

These are 6 x 6 (two-atom cell) Hermitian problems, a few per mode: host
work beside the GPU mode solve.  ``PrimitiveCell`` evaluates all
candidates of a batch of modes at once (stacked matrices, batched eigh).
"""
from __future__ import annotations

import numpy as np

PI = 3.141592653589793238   # negf/util.f90:5
_LAT125 = np.array([(i1, i2, i3) for i1 in range(-2, 3) for i2 in range(-2, 3) for i3 in range(-2, 3)],
                   dtype=np.float64)


def zone_flags(a, ks, chunk=4096):
    """Per row of ks: 2 when the two nearest points of the lattice a (rows)
    are equally near within 1e-5 (zone boundary), 1 when the origin is the
    nearest, 0 otherwise (negf/util.f90:589-638, 125 lattice points)."""
    ks = np.atleast_2d(np.asarray(ks, dtype=np.float64))
    lat = _LAT125 @ a
    out = np.zeros(ks.shape[0], dtype=np.int64)
    for s0 in range(0, ks.shape[0], chunk):
        part = ks[s0:s0 + chunk]
        d = part[:, None, :] - lat[None]
        dist = np.einsum("kij,kij->ki", d, d)
        first = np.argmin(dist, axis=1)
        rows = np.arange(part.shape[0])
        dmin = dist[rows, first]
        flag = np.where(np.abs(dist[:, 62] - dmin) < 1.0e-5, 1, 0)   # index 62: the origin
        dist[rows, first] = np.inf                                    # second smallest next
        out[s0:s0 + chunk] = np.where(np.abs(dist.min(axis=1) - dmin) < 1.0e-5, 2, flag)
    return out


class PrimitiveCell:
    """Primitive cell of a lead: the QE force constants folded onto its
    atoms, its reciprocal vectors and the unit cell's.

    qe: dict(pos, cell, fc (3,3,nat,nat,nx,ny,nz), rws, rd and nxyz or
    nx/ny/nz) of the QE force-constant file, as qe_input.read_qe_fc gives it; latvec (3x3 rows) and
    scaled (natoms_uc, 3) with species (1-based) and the lattice constant of
    the primitive-cell input (pc1.fdf style; the vectors are turned by
    pi/4 about z as negf/input.f90:617 does); mass_no: species masses;
    reci_uc: unit-cell reciprocal vectors (rows); l: max(n_bloch_x,
    n_bloch_y)."""

    def __init__(self, qe, latvec, scaled, species, lscale, mass_no, reci_uc, l):
        c, s = np.cos(PI / 4.0), np.sin(PI / 4.0)
        lat = np.asarray(latvec, dtype=np.float64) * lscale
        lat = np.stack([lat[:, 0] * c - lat[:, 1] * s, lat[:, 0] * s + lat[:, 1] * c, lat[:, 2]], axis=1)
        pos_uc = np.asarray(scaled, dtype=np.float64) @ lat
        inv = np.linalg.inv(lat)
        crys = pos_uc @ inv
        self.natoms = int(np.all((crys < 0.999) & (crys > -0.001), axis=1).sum())
        self.recivec = 2 * PI * inv.T
        self.reci_uc = np.asarray(reci_uc, dtype=np.float64)
        self.l = int(l)
        mass = np.asarray(mass_no, dtype=np.float64)[np.asarray(species) - 1]
        self._terms(qe, mass)
        self.zone_radius2 = (0.5 * np.linalg.norm(self.recivec, axis=1).sum() + 1.0e-3) ** 2
        g = np.arange(-self.l, self.l + 1, dtype=np.float64)
        self.gshift = np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(-1, 3) @ self.reci_uc

    def _terms(self, qe, mass):
        pos, cell, fc, rws, rd = qe["pos"], qe["cell"], qe["fc"], qe["rws"], qe["rd"]
        nx, ny, nz = (int(x) for x in (qe["nxyz"] if "nxyz" in qe else (qe["nx"], qe["ny"], qe["nz"])))
        n = np.arange
        abc = np.stack(np.meshgrid(n(-2 * nx, 2 * nx + 1), n(-2 * ny, 2 * ny + 1), n(-2 * nz, 2 * nz + 1),
                                   indexing="ij"), axis=-1).reshape(-1, 3).astype(np.float64)
        ivcell = np.linalg.inv(cell)
        na = self.natoms
        blocks = [[[] for _ in range(na)] for _ in range(na)]
        bonds = [[[] for _ in range(na)] for _ in range(na)]
        for i in range(na):
            for j in range(pos.shape[0]):
                dr = pos[j] - pos[i] - abc @ cell
                df = dr @ rws.T - rd[None, :]
                ok = ~(df > 1.0e-5).any(axis=1)
                nreq = 1 + (np.abs(df) <= 1.0e-5).sum(axis=1)
                cells = np.rint((dr - (pos[j] - pos[i])) @ ivcell).astype(np.int64)   # = -(a, b, c)
                for t in np.nonzero(ok)[0]:
                    # the cell (a, b, c) of the term; the reference's 1-based
                    # wrap mod(a + 1, nx) (raised to nx when <= 0) is a mod nx
                    ia, ib, ic = -cells[t]
                    blk = fc[:, :, i, j, ia % nx, ib % ny, ic % nz] / nreq[t] / np.sqrt(mass[i] * mass[j])
                    blocks[i][j % na].append(blk)
                    bonds[i][j % na].append(dr[t])
        # all terms stacked: the phases of a batch of k are one exp, each
        # (i, j) block one (B x T_ij) x (T_ij x 9) product
        self.bonds = np.concatenate([np.array(bonds[i][j]).reshape(-1, 3) for i in range(na) for j in range(na)])
        self.spans, t = [], 0
        for i in range(na):
            for j in range(na):
                nt = len(blocks[i][j])
                self.spans.append((i, j, t, t + nt, np.array(blocks[i][j]).reshape(nt, 9).astype(np.complex128)))
                t += nt

    def dynamical(self, ks):
        """(B, 3 na, 3 na) Hermitised dynamical matrices at the rows of ks."""
        ks = np.atleast_2d(np.asarray(ks, dtype=np.float64))
        return self._from_phases(np.exp(1j * (ks @ self.bonds.T)))

    def _from_phases(self, ph):
        na = self.natoms
        out = np.zeros((ph.shape[0], 3 * na, 3 * na), dtype=np.complex128)
        for i, j, t0, t1, blk in self.spans:
            out[:, 3 * i:3 * i + 3, 3 * j:3 * j + 3] = (ph[:, t0:t1] @ blk).reshape(-1, 3, 3)
        return 0.5 * (out + np.conj(np.swapaxes(out, 1, 2)))

    def bands(self, ks, step=1.0e-5):
        """Eigenvalues (ascending) and band velocities (central differences
        of D with step 1e-5) at the rows of ks."""
        ks = np.atleast_2d(np.asarray(ks, dtype=np.float64))
        ph = np.exp(1j * (ks @ self.bonds.T))
        eigs, evs = np.linalg.eigh(self._from_phases(ph))
        vel = np.zeros(eigs.shape + (3,))
        for d in range(3):
            # exp(i (k +- step e_d).r) = exp(i k.r) exp(+- i step r_d)
            shift = np.exp(1j * step * self.bonds[:, d])
            dh = (self._from_phases(ph * shift) - self._from_phases(ph * np.conj(shift))) / (2.0 * step)
            proj = np.einsum("bim,bij,bjm->bm", np.conj(evs), dh, evs)
            vel[:, :, d] = np.real(proj) / (2 * np.sqrt(np.abs(eigs)))
        return eigs, vel

    def unfold(self, E, ks):
        """(k_pc, v_pc) for modes with unfolded wavevectors ks (rows) at the
        energies E (omega^2), zeros where no candidate matches.  All
        candidates of all modes are solved in one batch."""
        ks = np.atleast_2d(np.asarray(ks, dtype=np.float64))
        nm = ks.shape[0]
        E = np.broadcast_to(np.asarray(E, dtype=np.float64), (nm,))
        kpc = np.zeros_like(ks)
        vpc = np.zeros_like(ks)
        if nm == 0:
            return kpc, vpc
        edge = zone_flags(self.reci_uc, ks) == 2
        allc = ks[:, None, :] + self.gshift[None]
        # a point of the primitive zone (boundary included) is within half the
        # summed lengths of the reciprocal vectors: only those are tested
        flat = allc.reshape(-1, 3)
        near = np.einsum("ij,ij->i", flat, flat) <= self.zone_radius2
        inside = np.zeros(flat.shape[0], dtype=bool)
        inside[near] = zone_flags(self.recivec, flat[near]) != 0
        inside = inside.reshape(nm, -1)
        inside[edge] = False
        own_n, g_n = np.nonzero(inside)               # grouped by mode, candidates in search order
        own_e = np.nonzero(edge)[0]
        owner = np.concatenate([own_e, own_n])
        cand = np.concatenate([ks[own_e], allc[own_n, g_n]])
        if owner.size == 0:
            return kpc, vpc
        eigs, vel = self.bands(cand)
        hit = np.abs(np.sqrt(E[owner])[:, None] - np.sqrt(np.abs(eigs))) < 1.0e-2
        any_hit = hit.any(axis=1)
        last = eigs.shape[1] - 1 - np.argmax(hit[:, ::-1], axis=1)      # the last matching band
        v_c = vel[np.arange(owner.size), last]
        ne = own_e.size
        # zone-boundary modes keep k; the velocity only when a band matches
        kpc[own_e] = ks[own_e]
        he = np.nonzero(any_hit[:ne])[0]
        vpc[own_e[he]] = v_c[he]
        # the others: among matching candidates the smallest |k| (first on
        # ties) and the velocity of the first
        idx = ne + np.nonzero(any_hit[ne:])[0]
        if idx.size:
            o = owner[idx]
            _, first = np.unique(o, return_index=True)
            vpc[o[first]] = v_c[idx[first]]
            norm = np.linalg.norm(cand[idx], axis=1)
            order = np.lexsort((np.arange(idx.size), norm, o))
            o_sorted = o[order]
            keep = np.ones(order.size, dtype=bool)
            keep[1:] = o_sorted[1:] != o_sorted[:-1]
            kpc[o_sorted[keep]] = cand[idx[order[keep]]]
        return kpc, vpc


def read_primitive_cell_fdf(path):
    """The primitive-cell input of a lead (negf/input.f90:579-627: the
    NumberOfAtoms and LatticeConstant tags, the LatticeVectors block and the
    AtomicScaledCoordinatesAndAtomicSpecies block).  Returns dict(latvec
    (3x3 rows, unscaled), scaled (natoms, 3), species (1-based), lscale)."""
    with open(path) as f:
        lines = f.read().splitlines()
    natoms, lscale = 0, 1.0
    latvec, scaled, species = None, [], []
    it = iter(lines)
    for line in it:
        tag = line.split()
        if not tag:
            continue
        if tag[0] == "NumberOfAtoms":
            natoms = int(tag[1])
        elif tag[0] == "LatticeConstant":
            lscale = float(tag[1])
        elif "%block LatticeVectors" in line:
            latvec = np.array([[float(x) for x in next(it).split()[:3]] for _ in range(3)])
        elif "%block AtomicScaledCoordinatesAndAtomicSpecies" in line:
            for _ in range(natoms):
                v = next(it).split()
                scaled.append([float(x) for x in v[:3]])
                species.append(int(v[3]))
    if latvec is None or len(scaled) != natoms:
        raise ValueError(f"{path}: incomplete primitive-cell input")
    return dict(latvec=latvec, scaled=np.array(scaled), species=np.array(species, dtype=np.int64), lscale=lscale)
