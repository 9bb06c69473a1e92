"""Pin the FP64 oracle against the reference's committed si-si outputs (CPU)."""
import os

import numpy as np
import pytest

from oracle import negf as N
from oracle import qe as Q
from tests.sisi_case import golden_close, sisi_blocks, sisi_params

REF = "/root/reference/examples/negf/si-si"


def test_fc_reader_matches_fc_qe_r_table(sisi):
    # fc_qe_r.dat is written by negf/fc.f90:211-248 with format 10F20.5
    ours = np.round(sisi["r_table_oracle"], 5)
    assert ours.shape == sisi["r_table_ref"].shape == (1024, 10)
    assert np.abs(ours - sisi["r_table_ref"]).max() < 1e-9


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference checkout not present")
def test_fixture_regenerates_from_reference(sisi):
    qe = Q.read_qe_fc(os.path.join(REF, "Si444.fc"), 8.3, 1)
    assert np.array_equal(qe["fc"], sisi["fc"])
    g = np.loadtxt(os.path.join(REF, "output", "transl_tot.dat"))
    assert np.array_equal(g[:, 1:], sisi["transl_tot"])
    perk = np.load(os.path.join(os.path.dirname(__file__), "golden", "sisi_perk.npz"))
    for ik in perk["k_index"]:
        g = np.loadtxt(os.path.join(REF, "output", f"mdl_specular_param_{int(ik) + 1:06d}.dat"), ndmin=2)
        assert np.array_equal(g, perk[f"mdl_{int(ik)}"])


def test_energy_and_k_grids(sisi):
    # the file holds e24.16 (16 significant digits)
    assert np.allclose(Q.energy_grid(61, 0.001, 15.5), sisi["E_transl_tot"], rtol=1e-15, atol=0)
    kg = Q.k_grid_in_ws(Q.k_grid(7, 7), sisi["cell_all"])
    assert np.array_equal(kg, sisi["kgrid"])
    assert kg.shape == (49, 3)


@pytest.mark.parametrize("ik", [0, 24])
def test_oracle_transmission_matches_reference(sisi, ik):
    b = sisi_blocks(sisi, ik)
    p = sisi_params(sisi)
    E = sisi["E"]
    zf = np.zeros(E.size, bool)
    zf[0] = True
    r = N.transport(E, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"], zero_first=zf)
    okl, adl, ql = golden_close(r["transl"], sisi["transl_tot"][:, ik])
    okr, adr, qr = golden_close(r["transr"], sisi["transr_tot"][:, ik])
    assert okl, (adl, ql)
    assert okr, (adr, qr)
    # the reference zeroes the first energy point (lesser.f90:802-807)
    assert r["transl"][0] == 0.0 and r["transr"][0] == 0.0


def test_oracle_decimation_iteration_cap():
    from phinfortran_gb300 import systems as S
    b, E, p = S.tb_ribbon(W=4, L=3, ne=5, disorder=0.0)
    g, it = N.decimate(E + 1j * 1e-6, b["HL"], N.H(b["HLv"]), b["HLv"], 1e-14, max_iter=3)
    assert it.max() <= 3
