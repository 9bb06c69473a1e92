"""Host input side of the phonon driver: the QE force-constant file, the
supercell, the mass profile and the omega / k grids, as the Fortran driver
prepares them before the transport loop.

* ``read_qe_fc``: negf/fc.f90:103-325 -- the QE ``.fc`` file (Ry/bohr^2)
  scaled to THz^2 amu, the r_cut zeroing of whole 3x3 blocks (with the
  fc_qe_r.dat table of nearest image distances), the acoustic sum rule on
  the self term and its symmetrisation, and the 124 Wigner-Seitz vectors
  of the force-constant supercell;
* ``build_supercell``: negf/fc.f90:291-322 (z layer outermost, then y,
  then x, then the QE basis atom);
* ``read_mass_profile`` / ``read_species_masses``: mass_profile.dat and the
  ChemicalSpeciesLabel block (negf/fc.f90:300-305, negf/input.f90:560-577,
  element masses negf/input.f90:410-440);
* ``energy_grid`` / ``k_grid`` / ``k_grid_in_ws``: negf/config.f90:153-216
  and negf/input.f90:475-518.

The unit constants are the reference's own, single-precision literals
included (bohr2ang = 0.529177 and the Ry/bohr^2 bracket are default-real
in negf/fc.f90), because the force constants, and so T, depend on them at
the 1e-8 level.
"""
from __future__ import annotations

import re

import numpy as np

PI = 3.141592653589793238            # negf/util.f90:5
ELE_VOLT = 1.609e-19                  # negf/util.f90:7
MASS_PROTON = 1.6726219e-27           # negf/util.f90:8
F32 = np.float32
BOHR2ANG = float(F32(0.529177))      # real(8) initialised from a default-real literal
RY_BOHR2 = float(F32(F32(13.605662285137) / (F32(0.529177249) * F32(0.529177249))))
FC_SCALE = ELE_VOLT / 1.0e-20 / MASS_PROTON / (1.0e12 * 2.0 * PI) ** 2 * RY_BOHR2
ELEMENT_MASS = {14: 28.0855, 32: 72.64, 33: 32.0971, 34: 31.0942, 35: 30.0913, 36: 29.0884}


def _num(tok):
    return float(tok.replace("D", "E").replace("d", "e"))


def read_qe_fc(path, r_cutoff, update_nbr=1):
    """dict(cell, pos, mass, nx, ny, nz, fc (3,3,nat,nat,nx,ny,nz) THz^2 amu,
    cell_sc, rws (124,3), rd (124,), r_table (rows of fc_qe_r.dat when
    update_nbr == 1))."""
    with open(path) as f:
        lines = f.read().splitlines()
    head = lines[0].split()
    ntype, nat = int(head[0]), int(head[1])
    scale = float(head[3]) * BOHR2ANG
    cell = np.array([[_num(t) for t in lines[1 + r].split()] for r in range(3)]) * scale
    species = {}
    for line in lines[4:4 + ntype]:
        m = re.match(r"\s*(\d+)\s+'([^']*)'", line)
        if m.group(2).strip() != "Si":          # negf/fc.f90:327-338 knows silicon only
            raise ValueError(f"{path}: element {m.group(2).strip()!r} is not known to the reader")
        species[int(m.group(1))] = float(F32(28.0855))
    atoms = [lines[4 + ntype + i].split() for i in range(nat)]
    pos = np.array([[_num(t) for t in a[2:5]] for a in atoms]) * scale
    mass = np.array([species[int(a[1])] for a in atoms])
    o = 4 + ntype + nat + 1                          # after the 'F' / 'T' line
    nx, ny, nz = (int(t) for t in lines[o].split())
    ncell = nx * ny * nz
    # blocks of one header line (a b ia ja) and ncell value lines (i j k value)
    body = np.array(" ".join(lines[o + 1:o + 1 + (nat * 3) ** 2 * (ncell + 1)]).replace("D", "E").split(),
                    dtype=np.float64).reshape((nat * 3) ** 2, 4 + 4 * ncell)
    fc = np.zeros((3, 3, nat, nat, nx, ny, nz))
    a, b, ia, ja = (body[:, t].astype(np.int64) - 1 for t in range(4))
    vals = body[:, 4:].reshape(-1, ncell, 4)
    ci, cj, ck = (vals[:, :, t].astype(np.int64) - 1 for t in range(3))
    fc[a[:, None], b[:, None], ia[:, None], ja[:, None], ci, cj, ck] = vals[:, :, 3] * FC_SCALE
    cell_sc = cell * np.array([nx, ny, nz])[:, None]
    r_table = None
    if update_nbr == 1:
        # nearest periodic image of every (ia, ja, cell) bond over 5^3 supercell shifts
        m = np.array([(p, q, r) for p in range(-2, 3) for q in range(-2, 3) for r in range(-2, 3)], float)
        cells = np.array([(p, q, r) for p in range(nx) for q in range(ny) for r in range(nz)], float)
        bond = pos[None, :, None, :] - pos[:, None, None, :] - (cells @ cell)[None, None]   # (ia, ja, cell, 3)
        img = bond[..., None, :] + (m @ cell_sc)[None, None, None]
        rmin = np.sqrt(np.einsum("...i,...i->...", img, img).min(axis=-1))               # (ia, ja, cell)
        blocks = fc.reshape(3, 3, nat, nat, ncell)
        r_table = np.concatenate([rmin.reshape(-1, 1),
                                  np.transpose(blocks, (2, 3, 4, 1, 0)).reshape(-1, 9)], axis=1)
        cut = rmin.reshape(nat, nat, nx, ny, nz) > r_cutoff
        fc[:, :, cut] = 0.0
    # acoustic sum rule on the self term (upper triangle), then its lower triangle mirrored
    idx = np.arange(nat)
    total = fc.sum(axis=(3, 4, 5, 6))                                  # (3, 3, nat)
    self_term = fc[:, :, idx, idx, 0, 0, 0]                            # (3, 3, nat)
    upper = np.triu(np.ones((3, 3), dtype=bool))[:, :, None]
    self_term = np.where(upper, self_term - total, self_term)
    self_term = np.where(upper, self_term, np.swapaxes(self_term, 0, 1))
    fc[:, :, idx, idx, 0, 0, 0] = self_term
    m = np.array([(p, q, r) for p in range(-2, 3) for q in range(-2, 3) for r in range(-2, 3)
                  if (p, q, r) != (0, 0, 0)], float)
    # m1 a1 + m2 a2 + m3 a3 and 0.5 |r|^2, summed in the reference's order
    rws = m[:, 0:1] * cell_sc[0] + m[:, 1:2] * cell_sc[1] + m[:, 2:3] * cell_sc[2]
    rd = 0.5 * (rws[:, 0] * rws[:, 0] + rws[:, 1] * rws[:, 1] + rws[:, 2] * rws[:, 2])
    return dict(cell=cell, pos=pos, mass=mass, nx=nx, ny=ny, nz=nz, fc=fc, cell_sc=cell_sc, rws=rws, rd=rd,
                r_table=r_table)


def build_supercell(qe, n_bloch_x, n_bloch_y, nz):
    """(cell_all, pos_all, idxall 0-based QE basis index) of the transport
    supercell."""
    cell, pos = qe["cell"], qe["pos"]
    nat = pos.shape[0]
    cell_all = cell * np.array([n_bloch_x, n_bloch_y, nz])[:, None]
    shifts = np.array([(x, y, z) for z in range(nz) for y in range(n_bloch_y) for x in range(n_bloch_x)], float)
    pos_all = (shifts @ cell)[:, None, :] + pos[None]
    return cell_all, pos_all.reshape(-1, 3), np.tile(np.arange(nat, dtype=np.int64), shifts.shape[0])


def read_mass_profile(path):
    """Species id of every supercell atom (count first)."""
    tok = open(path).read().split()
    return np.array(tok[1:1 + int(tok[0])], dtype=np.int64)


def read_species_masses(fdf_path, mass_only=0, mass_ratio=1.0):
    """mass_no(:) of the ChemicalSpeciesLabel block (element masses as the
    reference's default-real literals; mass_only = 1 gives Ge the Si mass
    times mass_ratio)."""
    lines = open(fdf_path).read().splitlines()
    ns = next(int(ln.split()[1]) for ln in lines if ln.split()[:1] == ["NumberOfSpecies"])
    start = next(i for i, ln in enumerate(lines) if "%block ChemicalSpeciesLabel" in ln)
    out = np.zeros(ns)
    for ln in lines[start + 1:start + 1 + ns]:
        sid, z = (int(t) for t in ln.split()[:2])
        if mass_only == 0:
            out[sid - 1] = float(F32(ELEMENT_MASS[z]))
        else:
            out[sid - 1] = {14: float(F32(28.0855)), 32: float(F32(28.0855)) * mass_ratio}[z]
    return out


def energy_grid(ne, emin, emax):
    """omega^2 grid: ((i - 1)/(ne - 1) emax)^2 with the first point emin^2."""
    if ne == 1:
        return np.array([emax ** 2])
    g = (np.arange(ne) / (ne - 1) * emax) ** 2
    g[0] = emin ** 2
    return g


def k_grid(mesh1, mesh2):
    """Centred fractional transverse mesh (mesh1 outer)."""
    i, j = np.meshgrid(np.arange(mesh1), np.arange(mesh2), indexing="ij")
    kg = np.zeros((mesh1 * mesh2, 3))
    kg[:, 0] = i.ravel() / mesh1 - 0.5 * (mesh1 - 1) / mesh1
    kg[:, 1] = j.ravel() / mesh2 - 0.5 * (mesh2 - 1) / mesh2
    if kg.shape[0] == 1:
        kg[0, :2] = 0.0
    return kg


def k_grid_in_ws(kg, latvec):
    """Fold every k into the in-plane Wigner-Seitz cell of the supercell
    (first minimum over the 5 x 5 in-plane shifts, i1 outer)."""
    a = 2 * PI * np.linalg.inv(latvec).T
    a[2] = 0.0
    nd = np.array([(p, q, 0.0) for p in range(-2, 3) for q in range(-2, 3)])
    d = (kg @ a)[:, None, :] - (nd @ a)[None]
    best = np.argmin(np.einsum("kij,kij->ki", d, d), axis=1)
    return kg - nd[best]
