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


def _sc_force_constants(nx, ny, nlay, k_bond):
    """Real-space central NN spring matrix of an nx*ny*nlay simple-cubic bar.

    Periodic in x and y (Gamma point of the transverse supercell).  k_bond is
    a callable (site_a, site_b, axis) -> spring constant.  Returns the dense
    (3N x 3N) force-constant matrix Phi with Phi_ii = -sum_j Phi_ij.
    """
    N = nx * ny * nlay

    def site(ix, iy, iz):
        return (iz * ny + iy % ny) * nx + ix % nx

    Phi = np.zeros((3 * N, 3 * N))
    for iz in range(nlay):
        for iy in range(ny):
            for ix in range(nx):
                a = site(ix, iy, iz)
                for axis, nb in ((0, (ix + 1, iy, iz)), (1, (ix, iy + 1, iz)), (2, (ix, iy, iz + 1))):
                    if nb[2] >= nlay:
                        continue
                    if axis == 0 and nx == 1 or axis == 1 and ny == 1:
                        continue
                    b = site(*nb)
                    kk = k_bond(a, b, axis)
                    # central force along the bond axis: only the (axis, axis) entry
                    Phi[3 * a + axis, 3 * b + axis] -= kk
                    Phi[3 * b + axis, 3 * a + axis] -= kk
                    Phi[3 * a + axis, 3 * a + axis] += kk
                    Phi[3 * b + axis, 3 * b + axis] += kk
    return Phi


def sc_phonon(nx=4, ny=4, L=20, k=1.0, mass_range=(1.0, 2.0), lead_mass=1.0, ne=256, eta=1e-5,
              convergence=1e-14, seed_index=1, bond_range=None):
    """Simple-cubic phonon bar with nearest-neighbour central springs.

    Device masses i.i.d. uniform in mass_range, leads lead_mass; optional
    per-bond springs uniform in bond_range.  Frequencies uniform on
    (0, omega_max], omega_max = 2 sqrt(k/m_lead) (top of the lead band);
    E = omega^2 with eta = 0, eta0 = eta and the reference's device factor 10.
    Returns (blocks, E, params, aux) with aux holding masses and springs.
    """
    rng = _rng(seed_index)
    nc = nx * ny
    n = 3 * nc
    # layers: 0 pad | 1 lead cell -1 | 2 lead cell 0 | 3..L+2 device |
    #         L+3 lead cell N+1 | L+4 lead cell N+2 | L+5 pad
    # (the pad layers give the lead cells their bulk onsite terms)
    nlay = L + 6
    d0 = 3
    masses = np.full(nlay * nc, float(lead_mass))
    masses[d0 * nc:(d0 + L) * nc] = rng.uniform(*mass_range, size=L * nc)
    springs = {}

    def kb(a, b, axis):
        if bond_range is None:
            return k
        la, lb = a // nc, b // nc
        if d0 <= la < d0 + L and d0 <= lb < d0 + L:
            key = (min(a, b), max(a, b), axis)
            if key not in springs:
                springs[key] = rng.uniform(*bond_range)
            return springs[key]
        return k

    Phi = _sc_force_constants(nx, ny, nlay, kb)
    m3 = np.repeat(masses, 3)
    D = Phi / np.sqrt(np.outer(m3, m3))

    def blk(i, j):
        return D[i * n:(i + 1) * n, j * n:(j + 1) * n].astype(np.complex128)

    HL, HLv = blk(1, 1), blk(1, 2)
    Hd = np.array([blk(d0 + i, d0 + i) for i in range(L)])
    Hdv = (np.array([blk(d0 + i, d0 + 1 + i) for i in range(L - 1)]) if L > 1
           else np.zeros((0, n, n), complex))
    Hld = blk(2, d0)
    Hrd = blk(d0 + L, d0 + L - 1)
    HR, HRv = blk(d0 + L + 1, d0 + L + 1), blk(d0 + L + 1, d0 + L)
    blocks = dict(HL=HL, HLv=HLv, HR=HR, HRv=HRv, Hd=Hd, Hdv=Hdv, Hld=Hld, Hrd=Hrd)
    wmax = 2.0 * np.sqrt(k / lead_mass)
    w = np.arange(1, ne + 1) / ne * wmax
    E = w ** 2
    params = dict(eta=0.0, eta0=eta, dev_factor=10.0, convergence=convergence)
    aux = dict(masses=masses, springs=springs, omega=w, omega_max=wmax)
    return blocks, E, params, aux
