"""Seeded synthetic block-tridiagonal systems of the benchmark workloads.

Each builder returns the tdb block set (HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd)
with the reference's orientation conventions (negf/dyn.f90:1482-2080):
HLv = H_{-1,0}, HRv = H_{N+2,N+1}, Hdv[i] = H_{i,i+1}, Hld = H_{0,1},
Hrd = H_{N+1,N}; plus the energy grid and the physics parameters the
reference's config file would hold.

Seeds follow numpy PCG64 with seed = 20261203 + workload index.
"""
from __future__ import annotations

import numpy as np

SEED0 = 20261203


def _rng(idx):
    return np.random.Generator(np.random.PCG64(SEED0 + idx))


def tb_ribbon(W=32, L=200, t=-1.0, disorder=0.5, ne=1024, emin=-4.2, emax=4.2, eta=1e-6,
              convergence=1e-14, seed_index=2):
    """Single-orbital nearest-neighbour square-lattice ribbon (electrons).

    Width W sites with open edges, hopping t, L device slices with Anderson
    onsite energies uniform in [-disorder, disorder]*|t|; pristine leads.
    The electron driver's fixed broadening (tb/surface.f90:216,
    tb/device.f90:390) maps to eta=0, eta0=eta, dev_factor=1; the energy
    grid is the linear one of tb/config.f90:210-216.
    """
    rng = _rng(seed_index)
    Hs = np.zeros((W, W), np.complex128)
    i = np.arange(W - 1)
    Hs[i, i + 1] = t
    Hs[i + 1, i] = t
    Vz = t * np.eye(W, dtype=np.complex128)
    eps = rng.uniform(-disorder, disorder, size=(L, W)) * abs(t)
    Hd = np.repeat(Hs[None], L, axis=0)
    Hd[:, np.arange(W), np.arange(W)] += eps
    Hdv = np.repeat(Vz[None], max(L - 1, 0), axis=0)
    blocks = dict(HL=Hs.copy(), HLv=Vz.copy(), HR=Hs.copy(), HRv=Vz.copy(), Hd=Hd, Hdv=Hdv,
                  Hld=Vz.copy(), Hrd=Vz.copy())
    if ne == 1:
        E = np.array([emax])
    else:
        E = emin + np.arange(ne) / (ne - 1) * (emax - emin)
    params = dict(eta=0.0, eta0=eta, dev_factor=1.0, convergence=convergence)
    return blocks, E, params


class ScBar:
    """Layout of a simple-cubic bar with periodic nx x ny cross-section.

    Layers: 0 pad | 1 lead cell -1 | 2 lead cell 0 | 3..L+2 device |
    L+3 lead cell N+1 | L+4 lead cell N+2 | L+5 pad (the pad layers give the
    lead cells their bulk onsite terms).  ``bonds`` lists every nearest-
    neighbour bond (site_a, site_b, axis); ``dev_bond`` marks the bonds with
    both ends in the device (the ones that carry their own spring).
    """

    def __init__(self, nx, ny, L):
        self.nx, self.ny, self.L = nx, ny, L
        self.nc = nx * ny
        self.n = 3 * self.nc
        self.nlay = L + 6
        self.d0 = 3
        nc = self.nc

        def site(ix, iy, iz):
            return (iz * ny + iy % ny) * nx + ix % nx

        bonds = []
        for iz in range(self.nlay):
            for iy in range(ny):
                for ix in range(nx):
                    a = site(ix, iy, iz)
                    for axis, nb in ((0, (ix + 1, iy, iz)), (1, (ix, iy + 1, iz)), (2, (ix, iy, iz + 1))):
                        if nb[2] >= self.nlay:
                            continue
                        if axis == 0 and nx == 1 or axis == 1 and ny == 1:
                            continue
                        bonds.append((a, site(*nb), axis))
        self.bonds = np.array(bonds, dtype=np.int64)
        la, lb = self.bonds[:, 0] // nc, self.bonds[:, 1] // nc
        d0, d1 = self.d0, self.d0 + L
        self.dev_bond = (la >= d0) & (la < d1) & (lb >= d0) & (lb < d1)
        self.dev_atoms = np.arange(d0 * nc, d1 * nc)

    def dynamical_matrix(self, masses, springs):
        """D = Phi / sqrt(m m) for per-atom masses and per-bond springs."""
        N = self.nlay * self.nc
        Phi = np.zeros((3 * N, 3 * N))
        a, b, ax = self.bonds[:, 0], self.bonds[:, 1], self.bonds[:, 2]
        ia, ib = 3 * a + ax, 3 * b + ax
        np.add.at(Phi, (ia, ib), -springs)
        np.add.at(Phi, (ib, ia), -springs)
        np.add.at(Phi, (ia, ia), springs)
        np.add.at(Phi, (ib, ib), springs)
        m3 = np.repeat(masses, 3)
        return Phi / np.sqrt(np.outer(m3, m3))

    def blocks(self, masses, springs):
        D = self.dynamical_matrix(masses, springs)
        n, d0, L = self.n, self.d0, self.L

        def blk(i, j):
            return D[i * n:(i + 1) * n, j * n:(j + 1) * n].astype(np.complex128)

        Hd = np.array([blk(d0 + i, d0 + i) for i in range(L)])
        Hdv = (np.array([blk(d0 + i, d0 + 1 + i) for i in range(L - 1)]) if L > 1
               else np.zeros((0, n, n), complex))
        return dict(HL=blk(1, 1), HLv=blk(1, 2), HR=blk(d0 + L + 1, d0 + L + 1), HRv=blk(d0 + L + 1, d0 + L),
                    Hd=Hd, Hdv=Hdv, Hld=blk(2, d0), Hrd=blk(d0 + L, d0 + L - 1))

    def sensitivity_matrix(self, M):
        """Dense GD (3N x 3N) with dF = Re sum_ab dD_ab GD_ab from the block
        sensitivities M of one q (M_B as returned by the adjoint: dF = Re Tr[dB M_B])."""
        n, d0, L = self.n, self.d0, self.L
        N3 = 3 * self.nlay * self.nc
        GD = np.zeros((N3, N3), np.complex128)

        def put(i, j, Mb):
            GD[i * n:(i + 1) * n, j * n:(j + 1) * n] += np.swapaxes(Mb, -1, -2)

        for i in range(L):
            put(d0 + i, d0 + i, M["Hd"][i])
        for i in range(L - 1):
            put(d0 + i, d0 + 1 + i, M["Hdv"][i])
        put(2, d0, M["Hld"])
        put(d0 + L, d0 + L - 1, M["Hrd"])
        return GD

    def parameter_gradient(self, GD, masses, springs):
        """(dF/dmasses (all atoms), dF/dsprings (all bonds)) from GD."""
        D = self.dynamical_matrix(masses, springs)
        P = np.real(D * GD)
        m3 = np.repeat(masses, 3)
        per_dof = -(P.sum(axis=1) + P.sum(axis=0)) / (2 * m3)
        gm = per_dof.reshape(-1, 3).sum(axis=1)
        a, b, ax = self.bonds[:, 0], self.bonds[:, 1], self.bonds[:, 2]
        ia, ib = 3 * a + ax, 3 * b + ax
        gk = np.real(-(GD[ia, ib] + GD[ib, ia]) / np.sqrt(masses[a] * masses[b])
                     + GD[ia, ia] / masses[a] + GD[ib, ib] / masses[b])
        return gm, gk


def sc_phonon(nx=4, ny=4, L=20, k=1.0, mass_range=(1.0, 2.0), lead_mass=1.0, ne=256, eta=1e-5,
              convergence=1e-14, seed_index=1, bond_range=None):
    """Simple-cubic phonon bar with nearest-neighbour central springs.

    Device masses i.i.d. uniform in mass_range, leads lead_mass; optional
    per-bond springs uniform in bond_range for the bonds inside the device.
    Frequencies uniform on (0, omega_max], omega_max = 2 sqrt(k/m_lead)
    (top of the lead band); E = omega^2 with eta = 0, eta0 = eta and the
    reference's device factor 10.  Returns (blocks, E, params, aux); aux
    holds the ScBar layout, masses and springs.
    """
    rng = _rng(seed_index)
    bar = ScBar(nx, ny, L)
    masses = np.full(bar.nlay * bar.nc, float(lead_mass))
    masses[bar.dev_atoms] = rng.uniform(*mass_range, size=bar.dev_atoms.size)
    springs = np.full(len(bar.bonds), float(k))
    if bond_range is not None:
        springs[bar.dev_bond] = rng.uniform(*bond_range, size=int(bar.dev_bond.sum()))
    blocks = bar.blocks(masses, springs)
    wmax = 2.0 * np.sqrt(k / lead_mass)
    w = np.arange(1, ne + 1) / ne * wmax
    E = w ** 2
    params = dict(eta=0.0, eta0=eta, dev_factor=10.0, convergence=convergence)
    aux = dict(bar=bar, masses=masses, springs=springs, omega=w, omega_max=wmax)
    return blocks, E, params, aux


def _diamond_layer(nc, a=1.0):
    """Atom positions of one layer: nc x nc conventional diamond cells,
    one cell thick along z (8 nc^2 atoms)."""
    fcc = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]], dtype=np.float64)
    basis = np.concatenate([fcc, fcc + 0.25])
    pos = [basis + np.array([ix, iy, 0.0]) for ix in range(nc) for iy in range(nc)]
    return np.concatenate(pos) * a


def _diamond_force_blocks(nc, kgrid, k1, k2, a=1.0, tol=1e-6):
    """Onsite (layer j, j) and coupling (layer j, j+1) force-constant blocks
    of a periodic nc x nc diamond slab with central first- and second-
    neighbour springs, Bloch-summed over the transverse images for every k
    (fractional units of the slab's transverse reciprocal vectors)."""
    pos = _diamond_layer(nc, a)
    na = pos.shape[0]
    d1, d2 = a * np.sqrt(3) / 4, a / np.sqrt(2)
    nk = kgrid.shape[0]
    F0 = np.zeros((nk, 3 * na, 3 * na), np.complex128)
    F1 = np.zeros((nk, 3 * na, 3 * na), np.complex128)
    self_term = np.zeros((na, 3, 3))
    for ix in (-1, 0, 1):
        for iy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                shift = np.array([ix * nc * a, iy * nc * a, dz * a])
                r = pos[None, :, :] + shift - pos[:, None, :]          # (a, b, 3)
                d = np.linalg.norm(r, axis=-1)
                kk = np.where(np.abs(d - d1) < tol, k1, np.where(np.abs(d - d2) < tol, k2, 0.0))
                ia, ib = np.nonzero(kk)
                if ia.size == 0:
                    continue
                e = r[ia, ib] / d[ia, ib][:, None]
                K = kk[ia, ib][:, None, None] * e[:, :, None] * e[:, None, :]   # (pairs, 3, 3)
                np.add.at(self_term, ia, K)
                if dz < 0:
                    continue
                ph = np.exp(2j * np.pi * (kgrid[:, 0] * ix + kgrid[:, 1] * iy))  # (nk,)
                tgt = F0 if dz == 0 else F1
                for p in range(ia.size):
                    A, B = 3 * ia[p], 3 * ib[p]
                    tgt[:, A:A + 3, B:B + 3] -= ph[:, None, None] * K[p][None]
    for A in range(na):
        F0[:, 3 * A:3 * A + 3, 3 * A:3 * A + 3] += self_term[A][None]
    return F0, F1


def diamond_phonon(nc=2, L=60, nk_side=8, ne=512, k1=1.0, k2=0.2, masses=(28.0, 72.6), block=10, eta=1e-5,
                   convergence=1e-14, kpoints=None):
    """Phonons of a diamond-lattice slab stack with a mass interface.

    Cross-section nc x nc conventional cells (n = 24 nc^2 DOF per layer, one
    cell thick), periodic transversally with Bloch wave vectors on an
    nk_side x nk_side grid centred as the reference's transverse mesh
    (negf/config.f90:153-175); central springs k1 (first neighbours) and k2
    (second neighbours).  Device layers alternate masses[0] / masses[1] in
    blocks of `block` layers; each lead takes the mass of the device block
    next to it.  Frequencies uniform on (0, omega_max] with omega_max the top
    of the left lead's spectrum; E = omega^2, eta = 0, eta0 = eta.
    ``kpoints`` selects a subset of the grid (indices).  Returns the
    q-stacked blocks, E, params and aux (kgrid, omega, n).
    """
    n1 = nk_side
    g = np.array([[(i / n1) - 0.5 * (n1 - 1) / n1, (j / n1) - 0.5 * (n1 - 1) / n1, 0.0]
                  for i in range(n1) for j in range(n1)])
    if n1 == 1:
        g[:] = 0.0
    if kpoints is not None:
        g = g[np.asarray(kpoints)]
    F0, F1 = _diamond_force_blocks(nc, g, k1, k2)
    n = F0.shape[-1]
    layer_mass = np.array([masses[(j // block) % 2] for j in range(L)], dtype=np.float64)
    mL, mR = layer_mass[0], layer_mass[-1]
    s = 1.0 / np.sqrt(layer_mass)
    Hd = F0[:, None] * (s ** 2)[None, :, None, None]
    Hdv = F1[:, None] * (s[:-1] * s[1:])[None, :, None, None] if L > 1 else np.zeros((g.shape[0], 0, n, n))
    blocks = dict(HL=F0 / mL, HLv=F1 / mL, HR=F0 / mR, HRv=np.conj(np.swapaxes(F1, -1, -2)) / mR,
                  Hd=Hd, Hdv=Hdv, Hld=F1 / np.sqrt(mL * layer_mass[0]),
                  Hrd=np.conj(np.swapaxes(F1, -1, -2)) / np.sqrt(layer_mass[-1] * mR))
    # top of the left lead's band at k = 0 of the first transverse point
    Hb = F0[0] + F1[0] + np.conj(F1[0].T)
    Hpi = F0[0] - F1[0] - np.conj(F1[0].T)
    wmax = np.sqrt(max(np.linalg.eigvalsh(Hb).max(), np.linalg.eigvalsh(Hpi).max()) / mL)
    w = wmax * np.arange(1, ne + 1) / ne
    params = dict(eta=0.0, eta0=eta, dev_factor=10.0, convergence=convergence)
    aux = dict(kgrid=g, omega=w, omega_max=wmax, n=n, layer_mass=layer_mass)
    return blocks, w ** 2, params, aux


def tb_ribbon3(W=256, L=1000, norb=3, onsite_sigma=0.3, hop_spread=0.1, ne=4096, emin=-4.2, emax=4.2, eta=1e-6,
               convergence=1e-14, seed_index=5, energies=None):
    """Multi-orbital nearest-neighbour square-lattice ribbon (electrons).

    Width W sites with open edges and `norb` orbitals per site (n = W norb
    per slice, orbital-major within a site).  Device slices: onsite energies
    N(0, onsite_sigma^2) per orbital and every bond's hopping 1 + U[-spread,
    spread] per orbital (orbital-diagonal); leads pristine (onsite 0,
    hopping 1).  eta = 0, eta0 = eta, dev_factor = 1 as in the electron
    driver; energies linear on [emin, emax] (``energies`` picks indices).
    """
    rng = _rng(seed_index)
    n = W * norb
    site = lambda i, o: i * norb + o

    def slab(tv):
        H = np.zeros((n, n), np.complex128)
        for i in range(W - 1):
            for o in range(norb):
                H[site(i, o), site(i + 1, o)] = tv[i, o]
                H[site(i + 1, o), site(i, o)] = tv[i, o]
        return H

    def coup(tz):
        return np.diag(tz.reshape(-1)).astype(np.complex128)

    ones_t = np.ones((W - 1, norb))
    Hs = slab(ones_t)
    Vz = coup(np.ones((W, norb)))
    Hd = np.empty((L, n, n), np.complex128)
    for j in range(L):
        Hd[j] = slab(1.0 + rng.uniform(-hop_spread, hop_spread, size=(W - 1, norb)))
        Hd[j][np.arange(n), np.arange(n)] += rng.normal(0.0, onsite_sigma, size=n)
    Hdv = np.empty((max(L - 1, 0), n, n), np.complex128)
    for j in range(L - 1):
        Hdv[j] = coup(1.0 + rng.uniform(-hop_spread, hop_spread, size=(W, norb)))
    blocks = dict(HL=Hs.copy(), HLv=Vz.copy(), HR=Hs.copy(), HRv=Vz.copy(), Hd=Hd, Hdv=Hdv, Hld=Vz.copy(),
                  Hrd=Vz.copy())
    E = emin + np.arange(ne) / max(ne - 1, 1) * (emax - emin)
    if energies is not None:
        E = E[np.asarray(energies)]
    params = dict(eta=0.0, eta0=eta, dev_factor=1.0, convergence=convergence)
    return blocks, E, params


# THz^2 per (eV/A^2 / amu): the unit factor of negf/dyn.f90:138
FC_TO_THZ2 = 1.609e-19 / 1.0e-20 / 1.6726219e-27 / (1.0e12 * 2.0 * 3.141592653589793238) ** 2


def sc_bar_binary_fc(nx=2, ny=2, L=6, a0=2.0, k=1.0, mass_range=(20.0, 40.0), lead_mass=28.0,
                     bond_range=(0.8, 1.2), seed_index=4):
    """The simple-cubic bar of ``sc_phonon`` (per-atom masses, per-bond
    springs in the device) written as the input of the binary
    force-constant path: the whole sandwich (L + 6 layers, ScBar layout) is
    one unit cell, periodic transversally (nx x ny) and along z, with one
    species per atom; fc (3 n_uc, 27 * 3 n_uc) in eV/A^2 holds -k e e^T
    for every bond to the neighbour's supercell image and the matching self
    terms (acoustic sum rule).  Springs in eV/A^2, masses in amu, positions
    in Angstrom (lattice constant a0).  Returns a dict with the arrays the
    reference holds (fc, positions, supercell positions, cells, masses,
    sizes) and ``bar_blocks``: the ScBar blocks of the same model in THz^2,
    which the full-Hamiltonian path must reproduce at k = 0."""
    rng = _rng(seed_index)
    bar = ScBar(nx, ny, L)
    nc, nlay = bar.nc, bar.nlay
    n_uc = nc * nlay
    masses = np.full(n_uc, float(lead_mass))
    masses[bar.dev_atoms] = rng.uniform(*mass_range, size=bar.dev_atoms.size)
    springs = np.full(len(bar.bonds), float(k))
    springs[bar.dev_bond] = rng.uniform(*bond_range, size=int(bar.dev_bond.sum())) * k
    idx = np.arange(n_uc)
    ix, iy, iz = idx % nx, (idx // nx) % ny, idx // nc
    pos = np.stack([ix * a0, iy * a0, iz * a0, idx + 1.0], axis=1)       # column 4: species (1-based)
    cell = np.diag([nx * a0, ny * a0, nlay * a0]).astype(np.float64)
    recivec = np.ascontiguousarray((2.0 * np.pi * np.linalg.inv(cell)).T)

    def sc(off, atom):   # fc supercell column atom (nfc = (1, 1, 1)), negf/input.f90:462-463
        return ((off[0] + 1) * 9 + (off[1] + 1) * 3 + 1 + off[2]) * n_uc + atom

    fc = np.zeros((3 * n_uc, 27 * 3 * n_uc))
    for (a, b, axis), s in zip(bar.bonds, springs):
        off = [0, 0, 0]
        if axis == 0 and ix[b] < ix[a]:
            off[0] = 1
        if axis == 1 and iy[b] < iy[a]:
            off[1] = 1
        neg = [-o for o in off]
        fc[3 * a + axis, 3 * sc(off, b) + axis] -= s
        fc[3 * b + axis, 3 * sc(neg, a) + axis] -= s
        fc[3 * a + axis, 3 * sc([0, 0, 0], a) + axis] += s
        fc[3 * b + axis, 3 * sc([0, 0, 0], b) + axis] += s
    pos_sc = np.zeros((27 * n_uc, 4))
    for i in (-1, 0, 1):
        for j in (-1, 0, 1):
            for kk in (-1, 0, 1):
                base = sc([i, j, kk], 0)
                pos_sc[base:base + n_uc, 0:3] = pos[:, 0:3] + np.array([i, j, kk], dtype=np.float64) @ cell
                pos_sc[base:base + n_uc, 3] = pos[:, 3]
    blocks = {key: v * FC_TO_THZ2 for key, v in bar.blocks(masses, springs).items()}
    n3 = 3 * nc
    return dict(fc=fc, pos=pos, pos_uc=pos, pos_sc=pos_sc, cell=cell, latvec_uc=cell, recivec=recivec,
                masses=masses, nbx=1, nby=1, n_uc=n_uc, nz=nlay, nfc=(1, 1, 1), r_cutoff=1.2 * a0,
                nl=n3, nr=n3, n_buffer_l=n3, n_buffer_r=n3, bar=bar, springs=springs, bar_blocks=blocks)


def sc_lead_binary_fc(nx=2, ny=2, a0=2.0, k=1.0, mass=28.0):
    """Lead principal layer of ``sc_bar_binary_fc`` as the reference's lead
    input: one layer (nx x ny atoms) as the unit cell, periodic in x, y and
    z (period a0), uniform springs k and mass; fc (3 nc, 27 * 3 nc) eV/A^2
    with the bonds of every atom to its +x, +y, +z neighbours (and their
    reverses) and the self terms."""
    nc = nx * ny
    idx = np.arange(nc)
    ix, iy = idx % nx, idx // nx
    pos = np.stack([ix * a0, iy * a0, np.zeros(nc), np.ones(nc)], axis=1)
    cell = np.diag([nx * a0, ny * a0, a0]).astype(np.float64)

    def sc(off, atom):
        return ((off[0] + 1) * 9 + (off[1] + 1) * 3 + 1 + off[2]) * nc + atom

    fc = np.zeros((3 * nc, 27 * 3 * nc))
    for a in range(nc):
        for axis in range(3):
            if axis == 0 and nx == 1 or axis == 1 and ny == 1:
                continue
            off = [0, 0, 0]
            if axis == 0:
                b = iy[a] * nx + (ix[a] + 1) % nx
                off[0] = 1 if ix[a] + 1 == nx else 0
            elif axis == 1:
                b = ((iy[a] + 1) % ny) * nx + ix[a]
                off[1] = 1 if iy[a] + 1 == ny else 0
            else:
                b = a
                off[2] = 1
            neg = [-o for o in off]
            fc[3 * a + axis, 3 * sc(off, b) + axis] -= k
            fc[3 * b + axis, 3 * sc(neg, a) + axis] -= k
            fc[3 * a + axis, 3 * sc([0, 0, 0], a) + axis] += k
            fc[3 * b + axis, 3 * sc([0, 0, 0], b) + axis] += k
    pos_sc = np.zeros((27 * nc, 4))
    for i in (-1, 0, 1):
        for j in (-1, 0, 1):
            for kk in (-1, 0, 1):
                base = sc([i, j, kk], 0)
                pos_sc[base:base + nc, 0:3] = pos[:, 0:3] + np.array([i, j, kk], dtype=np.float64) @ cell
                pos_sc[base:base + nc, 3] = 1.0
    recivec = np.ascontiguousarray((2.0 * np.pi * np.linalg.inv(cell)).T)
    return dict(fc=fc, pos=pos, pos_sc=pos_sc, cell=cell, recivec=recivec, masses=np.full(nc, float(mass)),
                nbx=1, nby=1, n_uc=nc, nfc=(1, 1, 1), r_cutoff=1.2 * a0)
