"""Generate tests/golden/sisi.npz from the reference's committed si-si example.

Run in a checkout that has the reference at /root/reference:

    python tests/golden/make_golden.py

The fixture holds (a) the processed force constants and supercell of
examples/negf/si-si (read by the oracle's restatement of negf/fc.f90), and
(b) the primitive-cell input pc1.fdf and the species masses, (c) the
reference's own committed outputs output/trans{l,r}_tot.dat,
trans{l,r}_{s,ns}.dat and refl{l,r}_{s,ns}.dat (61 omega^2 x 49 k), so the
GPU tests can check parity on a machine without the reference checkout;
tests/golden/sisi_output_head.txt, the first rows of those tables
verbatim, which pin the text format of the output writer; and
tests/golden/sisi_perk.npz / sisi_perk_head.txt, the per-k mode files
(output/*_specular_param_*.dat) of three k points.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import qe as Q  # noqa: E402

REF = "/root/reference/examples/negf/si-si"


def main(out=os.path.join(HERE, "sisi.npz")):
    qe = Q.read_qe_fc(os.path.join(REF, "Si444.fc"), r_cutoff=8.3, update_nbr=1)
    cell_all, pos_all, idxall = Q.build_supercell(qe, 2, 2, 8)
    mass_id = Q.read_mass_profile(os.path.join(REF, "mass_profile.dat"))
    mass_no = Q.read_species_masses(os.path.join(REF, "trans_input.fdf"))
    mass_all = mass_no[mass_id - 1]
    kg = Q.k_grid_in_ws(Q.k_grid(7, 7), cell_all)
    E = Q.energy_grid(61, 0.001, 15.5)
    gold = {}
    for name in ["transl_tot", "transr_tot", "transl_s", "transl_ns", "transr_s", "transr_ns",
                 "refll_s", "refll_ns", "reflr_s", "reflr_ns"]:
        a = np.loadtxt(os.path.join(REF, "output", name + ".dat"))
        gold[name] = a[:, 1:]
        gold["E_" + name] = a[:, 0]
    r_table = np.loadtxt(os.path.join(REF, "fc_qe_r.dat"))
    # primitive-cell input of both leads (config: left/right_primitive_cell_input = pc1.fdf)
    pc = {}
    with open(os.path.join(REF, "pc1.fdf")) as g:
        lines = g.read().splitlines()
    for i, line in enumerate(lines):
        if line.startswith("LatticeConstant"):
            pc["pc_lscale"] = float(line.split()[1])
        if "%block LatticeVectors" in line:
            pc["pc_latvec"] = np.array([[float(x) for x in lines[i + 1 + r].split()] for r in range(3)])
        if "%block AtomicScaledCoordinatesAndAtomicSpecies" in line:
            rows = [lines[i + 1 + r].split() for r in range(4)]
            pc["pc_scaled"] = np.array([[float(x) for x in r[:3]] for r in rows])
            pc["pc_species"] = np.array([int(r[3]) for r in rows])
    mass_no_all = Q.read_species_masses(os.path.join(REF, "trans_input.fdf"))
    np.savez_compressed(
        out, fc=qe["fc"], cell=qe["cell"], pos=qe["pos"], mass=qe["mass"],
        nxyz=np.array([qe["nx"], qe["ny"], qe["nz"]]), cell_sc=qe["cell_sc"], rws=qe["rws"], rd=qe["rd"],
        cell_all=cell_all, pos_all=pos_all, idxall=idxall, mass_all=mass_all, kgrid=kg, E=E,
        r_table_ref=r_table, r_table_oracle=qe["r_table"],
        # config of examples/negf/si-si/config
        eta=1.0e-8, eta0=1.0e-9, convergence=1.17e-14, dev_factor=10.0,
        n_bloch=np.array([2, 2]), nz=8, buffer=16, period=16, nlayer=2, natm_layer=16,
        mass_no=mass_no_all, **pc, **gold)
    print("wrote", out)


TABLES = ["transl_s", "transl_ns", "refll_s", "refll_ns", "transr_s", "transr_ns", "reflr_s", "reflr_ns",
          "transl_tot", "transr_tot"]


def text_heads(out=os.path.join(HERE, "sisi_output_head.txt"), nlines=3):
    """Verbatim first rows of the ten output tables (the text format of
    negf/write_data.f90:340-497), one '# name' header before each."""
    with open(out, "w") as f:
        for name in TABLES:
            with open(os.path.join(REF, "output", name + ".dat")) as g:
                rows = [next(g) for _ in range(nlines)]
            f.write(f"# {name}\n")
            f.writelines(rows)
    print("wrote", out)


PERK_FILES = ["left", "right", "tlr", "trl", "mdl", "mdr"]
PERK_K = [0, 10, 37]   # 0-based k indices whose per-k mode files are kept


def perk(out=os.path.join(HERE, "sisi_perk.npz"), head=os.path.join(HERE, "sisi_perk_head.txt"), nlines=3):
    """The reference's per-k mode files (negf/write_data.f90:3-176) of a few
    k points, parsed (rows of count, E, k, k_pc, v_pc, sums), and the first
    rows of the k = 1 files verbatim (their text format)."""
    arrs = {}
    with open(head, "w") as h:
        for name in PERK_FILES:
            for ik in PERK_K:
                path = os.path.join(REF, "output", f"{name}_specular_param_{ik + 1:06d}.dat")
                arrs[f"{name}_{ik}"] = np.loadtxt(path, ndmin=2)
                if ik == 0:
                    with open(path) as g:
                        rows = [next(g) for _ in range(nlines)]
                    h.write(f"# {name}\n")
                    h.writelines(rows)
    np.savez_compressed(out, k_index=np.array(PERK_K), **arrs)
    print("wrote", out, head)


if __name__ == "__main__":
    main()
    text_heads()
    perk()
