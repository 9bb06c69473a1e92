"""Restatement of the phonon input side (oracle; tests only).

* ``read_qe_fc``   -- negf/fc.f90:103-325 (QE .fc reader, unit conversion,
                      r_cut zeroing with the fc_qe_r.dat table, acoustic sum
                      rule, 124 Wigner-Seitz vectors, supercell positions).
* ``energy_grid``  -- negf/config.f90:201-216 (omega^2 grid, first point emin^2).
* ``k_grid``       -- negf/config.f90:153-188 (centred transverse mesh).
* ``k_grid_in_ws`` -- negf/input.f90:475-518 (fold into the first zone).
* ``element_mass`` -- negf/input.f90:410-440; ``ele_mass`` fc.f90:327-338.

Arrays keep the reference's 1-based meaning but numpy 0-based storage:
``fc[a, b, iat, jat, i, j, k]`` is fc_qe(a+1, b+1, iat+1, jat+1, i+1, j+1, k+1).
"""
from __future__ import annotations

import math
import re

import numpy as np

PI = 3.141592653589793238          # negf/util.f90:5
ELE_VOLT = 1.609e-19                # negf/util.f90:7 (sic)
MASS_PROTON = 1.6726219e-27         # negf/util.f90:8

def _f32(x):
    """A default-real (single precision) Fortran literal promoted to real(8)."""
    return float(np.float32(x))


# negf/fc.f90:127 declares ``real(kind=8) :: bohr2ang = 0.529177`` -- a
# single-precision literal, so the stored value is float32(0.529177).
BOHR2ANG = _f32(0.529177)

# negf/fc.f90:204-206: eV/A^2 -> THz^2 amu, times Ry/bohr^2 -> eV/A^2.  The
# bracket ``(13.605662285137/0.529177249**2)`` holds single-precision
# literals and is evaluated in single precision.
_RY_BOHR2 = float(np.float32(np.float32(13.605662285137)
                             / (np.float32(0.529177249) * np.float32(0.529177249))))
FC_SCALE = ELE_VOLT / 1.0e-20 / MASS_PROTON / (1.0e12 * 2.0 * PI) ** 2 * _RY_BOHR2


def ele_mass(label):
    """negf/fc.f90:327-338: only silicon is known."""
    if label.strip() == "Si":
        return _f32(28.0855)
    raise ValueError(f"ele_mass: unknown element {label!r} (reference knows only Si)")


def element_mass(z, mass_only=0, mass_ratio=1.0):
    """negf/input.f90:410-440 (single-precision literals, as in the source)."""
    if mass_only == 0:
        table = {14: 28.0855, 32: 72.64, 33: 32.0971, 34: 31.0942,
                 35: 30.0913, 36: 29.0884}
        return _f32(table[z])
    return {14: _f32(28.0855), 32: _f32(28.0855) * mass_ratio}[z]


def _floats(line):
    return [float(x.replace("D", "E").replace("d", "e")) for x in line.split()]


def read_qe_fc(path, r_cutoff, update_nbr=1):
    """Read a QE ``.fc`` file as negf/fc.f90:103-325 does.

    Returns a dict: cell (3x3, rows = vectors, Angstrom), pos (nat,3),
    mass (nat,), nx, ny, nz, fc (3,3,nat,nat,nx,ny,nz) in THz^2 amu,
    cell_sc, rws (124,3), rd (124,), and ``r_table`` -- the rows the
    reference writes to fc_qe_r.dat (rmin followed by the 9 fc values in
    Fortran column order) when update_nbr == 1.
    """
    with open(path) as f:
        lines = f.read().splitlines()
    it = iter(lines)
    head = next(it).split()
    ntype, nat, _ibrav = int(head[0]), int(head[1]), int(head[2])
    celldm = [float(x) for x in head[3:9]]
    cell = np.array([_floats(next(it)) for _ in range(3)], dtype=np.float64)
    mass_ele = np.zeros(ntype)
    for i in range(ntype):
        m = re.match(r"\s*(\d+)\s+'([^']*)'\s+(\S+)", next(it))
        mass_ele[int(m.group(1)) - 1] = ele_mass(m.group(2))
    pos = np.zeros((nat, 3))
    mass = np.zeros(nat)
    for i in range(nat):
        v = next(it).split()
        pos[i] = [float(x) for x in v[2:5]]
        mass[i] = mass_ele[int(v[1]) - 1]
    scale = celldm[0] * BOHR2ANG
    pos = pos * scale
    cell = cell * scale
    next(it)                                  # 'F' / 'T' label line
    nx, ny, nz = (int(x) for x in next(it).split())
    cell_sc = np.array([nx * cell[0], ny * cell[1], nz * cell[2]])
    fc = np.zeros((3, 3, nat, nat, nx, ny, nz))
    for _ in range((nat * 3) ** 2):
        a, b, ia, ja = (int(x) for x in next(it).split())
        for _ in range(nx * ny * nz):
            v = next(it).split()
            i, j, k = int(v[0]), int(v[1]), int(v[2])
            fc[a - 1, b - 1, ia - 1, ja - 1, i - 1, j - 1, k - 1] = float(v[3]) * FC_SCALE
    r_table = []
    if update_nbr == 1:
        # cutoff radius (fc.f90:211-248): loop order iatm, jatm, j, k, l
        m = np.array([(m1, m2, m3) for m1 in range(-2, 3) for m2 in range(-2, 3)
                      for m3 in range(-2, 3)], dtype=np.float64)
        shifts = m @ cell_sc
        for ia in range(nat):
            for ja in range(nat):
                for j in range(nx):
                    for k in range(ny):
                        for l in range(nz):
                            base = pos[ja] - pos[ia] - np.array([j, k, l], float) @ cell
                            rmin = np.sqrt(((base[None, :] + shifts) ** 2).sum(axis=1)).min()
                            r_table.append([rmin] + list(fc[:, :, ia, ja, j, k, l].T.ravel()))
                            if rmin > r_cutoff:
                                fc[:, :, ia, ja, j, k, l] = 0.0
    # acoustic sum rule (fc.f90:250-258)
    for a in range(3):
        for b in range(a, 3):
            for idx in range(nat):
                fc[a, b, idx, idx, 0, 0, 0] = (-fc[a, b, idx].sum()
                                                + fc[a, b, idx, idx, 0, 0, 0])
    # permutation symmetry of the self term (fc.f90:260-266)
    for a in range(3):
        for b in range(a + 1):
            for idx in range(nat):
                fc[a, b, idx, idx, 0, 0, 0] = fc[b, a, idx, idx, 0, 0, 0]
    # Wigner-Seitz vectors (fc.f90:271-289)
    rws = []
    for m1 in range(-2, 3):
        for m2 in range(-2, 3):
            for m3 in range(-2, 3):
                if m1 == 0 and m2 == 0 and m3 == 0:
                    continue
                rws.append(cell_sc[0] * m1 + cell_sc[1] * m2 + cell_sc[2] * m3)
    rws = np.array(rws)
    rd = 0.5 * (rws * rws).sum(axis=1)
    return dict(cell=cell, pos=pos, mass=mass, nx=nx, ny=ny, nz=nz, fc=fc,
                cell_sc=cell_sc, rws=rws, rd=rd, r_table=np.array(r_table))


def build_supercell(qe, n_bloch_x, n_bloch_y, nz):
    """Supercell layout of negf/fc.f90:291-322.

    Atom order: z layer outermost, then y, then x, then the QE basis atom.
    Returns (cell_all, pos_all, idxall (0-based basis index)).
    """
    cell = qe["cell"]
    nat = qe["pos"].shape[0]
    cell_all = np.array([n_bloch_x * cell[0], n_bloch_y * cell[1], nz * cell[2]])
    pos_all, idxall = [], []
    for m1 in range(nz):
        for m2 in range(n_bloch_y):
            for m3 in range(n_bloch_x):
                for i in range(nat):
                    pos_all.append(qe["pos"][i] + np.array([m3, m2, m1], float) @ cell)
                    idxall.append(i)
    return cell_all, np.array(pos_all), np.array(idxall, dtype=np.int64)


def read_mass_profile(path):
    """mass_profile.dat as read at negf/fc.f90:300-305 (count, then species ids)."""
    with open(path) as f:
        vals = f.read().split()
    n = int(vals[0])
    return np.array([int(v) for v in vals[1:1 + n]], dtype=np.int64)


def read_species_masses(fdf_path, mass_only=0, mass_ratio=1.0):
    """mass_no(:) from the ChemicalSpeciesLabel block (negf/input.f90:560-577)."""
    with open(fdf_path) as f:
        lines = f.read().splitlines()
    nspecies = None
    for ln in lines:
        parts = ln.split()
        if parts and parts[0] == "NumberOfSpecies":
            nspecies = int(parts[1])
    mass_no = np.zeros(nspecies)
    for i, ln in enumerate(lines):
        if "%block ChemicalSpeciesLabel" in ln:
            for j in range(nspecies):
                v = lines[i + 1 + j].split()
                mass_no[int(v[0]) - 1] = element_mass(int(v[1]), mass_only, mass_ratio)
    return mass_no


def energy_grid(ne, emin, emax):
    """omega^2 grid of negf/config.f90:201-210."""
    if ne == 1:
        return np.array([emax ** 2])
    g = ((np.arange(ne) / (ne - 1)) * emax) ** 2
    g[0] = emin ** 2
    return g


def energy_grid_tb(ne, emin, emax):
    """Linear energy grid of tb/config.f90:210-216."""
    if ne == 1:
        return np.array([emax])
    return emin + np.arange(ne) / (ne - 1) * (emax - emin)


def k_grid(mesh1, mesh2):
    """Centred transverse mesh of negf/config.f90:153-176 (fractional)."""
    nk = mesh1 * mesh2
    kg = np.zeros((nk, 3))
    n = 0
    for i in range(mesh1):
        for j in range(mesh2):
            kg[n, 0] = i / mesh1
            kg[n, 1] = j / mesh2
            n += 1
    kg[:, 0] -= 0.5 * (mesh1 - 1) / mesh1
    kg[:, 1] -= 0.5 * (mesh2 - 1) / mesh2
    if nk == 1:
        kg[0, :2] = 0.0
    return kg


def k_grid_in_ws(kg, latvec):
    """negf/input.f90:475-518; ``latvec`` rows are the supercell vectors."""
    recivec = 2 * PI * np.linalg.inv(latvec).T
    a = recivec.copy()
    a[2, :] = 0.0
    out = kg.copy()
    nd = np.array([(i1, i2, 0.0) for i1 in range(-2, 3) for i2 in range(-2, 3)])
    for i in range(kg.shape[0]):
        kp = kg[i] @ a
        d = kp[None, :] - nd @ a
        dist = (d * d).sum(axis=1)
        out[i] = kg[i] - nd[int(np.argmin(dist))]
    return out


def ceil_div(a, b):
    return int(math.ceil(a / b))
