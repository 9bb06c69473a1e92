"""The package's host input side (phinfortran_gb300.qe_input) against the
oracle's restatement of negf/fc.f90, negf/config.f90 and negf/input.f90,
and against the si-si fixture (CPU)."""
import os

import numpy as np
import pytest

from oracle import qe as Q
from phinfortran_gb300 import qe_input as P

REF = "/root/reference/examples/negf/si-si"


def synthetic_fc(path, nat=2, n=(2, 2, 3), seed=5):
    """A small QE force-constant file: two Si atoms, a 2x2x3 supercell."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    out = [f"  1    {nat}  0  6.2000000  0.0000000  0.0000000  0.0000000  0.0000000  0.0000000",
           "      1.000000000    0.000000000    0.000000000",
           "      0.000000000    1.000000000    0.000000000",
           "      0.000000000    0.000000000    1.414213562",
           "           1  'Si '    25598.3672624059     ",
           "    1    1      0.0000000000      0.0000000000      0.0000000000",
           "    2    1      0.0000000000      0.5000000000      0.3535533906",
           " F", f"   {nx}   {ny}   {nz}"]
    for ja in range(nat):
        for ia in range(nat):
            for b in range(3):
                for a in range(3):
                    out.append(f"   {a + 1}   {b + 1}   {ia + 1}   {ja + 1}")
                    for k in range(nz):
                        for j in range(ny):
                            for i in range(nx):
                                out.append(f"   {i + 1}   {j + 1}   {k + 1}  {rng.normal() * 1e-2: .11E}")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


@pytest.mark.parametrize("r_cut", [3.0, 100.0])
def test_reader_matches_oracle_on_synthetic_file(tmp_path, r_cut):
    path = str(tmp_path / "x.fc")
    synthetic_fc(path)
    a, b = Q.read_qe_fc(path, r_cut, 1), P.read_qe_fc(path, r_cut, 1)
    for k in ("cell", "pos", "mass", "fc", "cell_sc", "rws", "rd"):
        assert np.array_equal(a[k], b[k]), k
    np.testing.assert_allclose(b["r_table"], a["r_table"], rtol=1e-13, atol=1e-13)
    if r_cut < 10:
        assert (b["fc"] == 0).any() and (b["fc"] != 0).any()


def test_supercell_and_grids_match_fixture(sisi):
    f = sisi
    qe = dict(cell=f["cell"], pos=f["pos"])
    cell_all, pos_all, idx = P.build_supercell(qe, 2, 2, int(f["nz"]))
    assert np.array_equal(cell_all, f["cell_all"]) and np.array_equal(pos_all, f["pos_all"])
    assert np.array_equal(idx, f["idxall"])
    assert np.array_equal(P.energy_grid(61, 0.001, 15.5), f["E"])
    assert np.array_equal(P.k_grid_in_ws(P.k_grid(7, 7), cell_all), f["kgrid"])
    for ne, m1, m2 in ((1, 1, 1), (5, 3, 4)):
        assert np.array_equal(P.energy_grid(ne, 0.2, 3.0), Q.energy_grid(ne, 0.2, 3.0))
        assert np.array_equal(P.k_grid(m1, m2), Q.k_grid(m1, m2))


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference checkout not present")
def test_reader_reproduces_fixture_from_reference_files(sisi):
    b = P.read_qe_fc(os.path.join(REF, "Si444.fc"), 8.3, 1)
    assert np.array_equal(b["fc"], sisi["fc"]) and np.array_equal(b["rws"], sisi["rws"])
    np.testing.assert_allclose(np.round(b["r_table"], 5), sisi["r_table_ref"], atol=1e-9)
    assert np.array_equal(P.read_species_masses(os.path.join(REF, "trans_input.fdf")), sisi["mass_no"])
    prof = P.read_mass_profile(os.path.join(REF, "mass_profile.dat"))
    assert np.array_equal(sisi["mass_no"][prof - 1], sisi["mass_all"])


def test_primitive_cell_takes_the_reader_dict(sisi):
    """unfold_pc.PrimitiveCell accepts read_qe_fc's dict (nx, ny, nz keys)
    as well as the fixture's nxyz."""
    from phinfortran_gb300.unfold_pc import PrimitiveCell
    from tests.sisi_case import sisi_primitive_cell
    f = sisi
    qe = dict(pos=f["pos"], cell=f["cell"], fc=f["fc"], rws=f["rws"], rd=f["rd"], nx=int(f["nxyz"][0]),
              ny=int(f["nxyz"][1]), nz=int(f["nxyz"][2]))
    a = PrimitiveCell(qe, f["pc_latvec"], f["pc_scaled"], f["pc_species"], float(f["pc_lscale"]), f["mass_no"],
                      2 * np.pi * np.linalg.inv(f["cell"]).T, 2)
    b = sisi_primitive_cell(f)
    k = np.array([[0.3, -0.2, 0.4], [0.0, 0.0, 0.1]])
    assert np.array_equal(a.dynamical(k), b.dynamical(k))
