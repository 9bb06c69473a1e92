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
