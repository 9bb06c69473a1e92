"""GPU per-mode outputs (pf_transport_tdb_modes_permode_dev) turned into
the reference's per-k mode files (write_specular / write_md,
negf/write_data.f90:3-176) -- with the primitive-cell columns of
unfold_pc -- and checked against the reference's files of three k
points, every column."""
import os

import numpy as np
import pytest

from phinfortran_gb300.modes import LeadGeometry, mode_rows, transport_tdb_modes
from phinfortran_gb300.output import write_mode_files
from tests.sisi_case import sisi_blocks, sisi_params, sisi_primitive_cell
from tests.test_mode_files_host import FILES, compare_rows

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_mode_files_against_reference(cuda_ready, sisi, tmp_path):
    f = sisi
    perk = np.load(os.path.join(HERE, "golden", "sisi_perk.npz"))
    ks = [int(k) for k in perk["k_index"]]
    nb = tuple(int(x) for x in f["n_bloch"])
    b, p = int(f["buffer"]), int(f["period"])
    geo = LeadGeometry.from_qe(f["pos_all"], f["cell"], f["cell_all"], nb, b, p, b, p)
    bl = [sisi_blocks(f, k) for k in ks]
    stacked = {name: np.stack([x[name] for x in bl]) for name in bl[0]}
    ne = f["E"].size
    E = np.tile(f["E"], len(ks))
    q = np.repeat(np.arange(len(ks)), ne).astype(np.int32)
    zf = np.tile((np.arange(ne) == 0).astype(np.int32), len(ks))
    cell = f["cell"]
    r = transport_tdb_modes(E, stacked, geo, f["kgrid"][ks], qidx=q, zero_flag=zf, lambda_eta=5e-3,
                            a_z_l=cell[2, 2], a_z_r=cell[2, 2], per_mode=True, **sisi_params(f))
    rows = mode_rows(r, geo, f["kgrid"][ks], E, qidx=q, pc=sisi_primitive_cell(f))
    # the per-mode rows add up to the eight sums of the same run
    for name, key, col in (("trl", "transr_s", 11), ("tlr", "transl_s", 11), ("left", "refll_s", 11),
                           ("right", "reflr_s", 11)):
        tot = np.array([sum(row[col] for row in rr) for _, rr in rows[name]])
        assert np.abs(tot - r[key]).max() <= 1e-12 + 1e-10 * np.abs(r[key]).max(), name
    for a, ik in enumerate(ks):
        for name in FILES:
            mine = [row for qq, rr in rows[name] if qq == a for row in rr]
            compare_rows(mine, perk[f"{name}_{ik}"], name.startswith("md"))
    # written files read back as the same rows
    write_mode_files(str(tmp_path), rows, k_index={a: ik + 1 for a, ik in enumerate(ks)})
    back = np.loadtxt(tmp_path / f"left_specular_param_{ks[0] + 1:06d}.dat", ndmin=2)
    compare_rows(back, perk[f"left_{ks[0]}"], False)
