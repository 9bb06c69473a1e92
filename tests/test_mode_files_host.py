"""The reference's per-k mode files (write_specular / write_md,
negf/write_data.f90:3-176, called at negf/velocity_mat.f90:3108-3128), CPU
side: the text format of the writer against the reference's own lines, the
oracle's rows against the reference's files of three k points, and the
append behaviour of the writer."""
import os

import numpy as np
import pytest

from oracle import modes as M
from oracle import unfold_pc as U
from phinfortran_gb300.output import mode_file_line, write_mode_files
from phinfortran_gb300.unfold_pc import read_primitive_cell_fdf
from tests.sisi_case import sisi_find_pc, sisi_primitive_cell
from tests.test_modes_host import oracle_point_sums

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = ("left", "right", "tlr", "trl", "mdl", "mdr")


@pytest.fixture(scope="module")
def perk():
    return np.load(os.path.join(HERE, "golden", "sisi_perk.npz"))


def compare_rows(A, B, md, pc=True):
    """Rows of one file against the reference's: the same energies, per
    energy the same number of rows and (after sorting by k, since the
    mode order inside an energy follows the eigen-solver) the same k within
    2e-9 (10-digit output), the sums within 5e-7 relative + 1e-12, the
    ratio r_s/r_t within 1e-9 where r_t > 1e-8 (below that it is the ratio
    of two rounding-level reflections); with ``pc`` the primitive-cell k
    within 1e-8 and velocity within 1e-6 relative + 1e-9."""
    A, B = np.asarray(A, dtype=np.float64), np.asarray(B, dtype=np.float64)

    def groups(a):
        d = {}
        for r in a:
            d.setdefault(round(float(r[1]), 8), []).append(r)
        return d

    ga, gb = groups(A), groups(B)
    assert sorted(ga) == sorted(gb)
    cols = [11, 12, 13, 14] if md else [11, 12]
    for e, rb in gb.items():
        key = lambda r: tuple(np.round(r[2:5], 6))
        a, b = np.array(sorted(ga[e], key=key)), np.array(sorted(rb, key=key))
        assert a.shape == b.shape, e
        assert sorted(a[:, 0]) == list(range(1, a.shape[0] + 1)), e
        assert np.abs(a[:, 2:5] - b[:, 2:5]).max() <= 2e-9, e
        assert (np.abs(a[:, cols] - b[:, cols]) <= 5e-7 * np.abs(b[:, cols]) + 1e-12).all(), e
        if not md:
            m = b[:, 12] > 1e-8
            assert (np.abs(a[m, 13] - b[m, 13]) <= 1e-9).all(), e
        if pc:
            assert np.abs(a[:, 5:8] - b[:, 5:8]).max() <= 1e-8, e
            assert (np.abs(a[:, 8:11] - b[:, 8:11]) <= 1e-6 * np.abs(b[:, 8:11]) + 1e-9).all(), e


def test_mode_file_line_matches_reference_text(perk):
    """Format 1000 of write_specular / write_md: I5 then E20.10."""
    with open(os.path.join(HERE, "golden", "sisi_perk_head.txt")) as f:
        text = f.read().split("# ")[1:]
    assert len(text) == len(FILES)
    for block in text:
        name, *lines = block.rstrip("\n").split("\n")
        rows = perk[f"{name}_0"]
        for i, line in enumerate(lines):
            assert mode_file_line(rows[i]) == line + "\n", (name, i)


@pytest.mark.parametrize("ik", [0, 37])
def test_oracle_mode_rows_match_reference(sisi, perk, ik):
    f = sisi
    cell = f["cell"]
    nb = tuple(int(x) for x in f["n_bloch"])
    reci_uc = 2 * np.pi * np.linalg.inv(cell).T
    geom = dict(ksc=f["kgrid"][ik], recivec=2 * np.pi * np.linalg.inv(f["cell_all"]).T, reci_uc_l=reci_uc,
                reci_uc_r=reci_uc, nb=nb)
    rows = {n: [] for n in FILES}
    find_pc = sisi_find_pc(f)
    for ie, (o, _) in enumerate(oracle_point_sums(f, ik, list(range(f["E"].size)))):
        for n, rr in M.mode_file_rows(f["E"][ie], o, geom, find_pc).items():
            rows[n] += rr
    for n in FILES:
        compare_rows(rows[n], perk[f"{n}_{ik}"], n.startswith("md"))


def test_primitive_cell_columns_match_reference(sisi, perk):
    """find_k_pc from the k and energy of every row of the reference's
    files (three k points, six files): the package's batched
    PrimitiveCell.unfold for all rows, the oracle's loop restatement for
    those of one file; both against the reference's k_pc and v_pc."""
    pc = sisi_primitive_cell(sisi)
    find_pc = sisi_find_pc(sisi)
    nonzero = 0
    for key in perk.files:
        if key == "k_index":
            continue
        r = perk[key]
        kp, vp = pc.unfold(r[:, 1] ** 2, r[:, 2:5])
        assert np.abs(kp - r[:, 5:8]).max() <= 1e-8, key
        assert (np.abs(vp - r[:, 8:11]) <= 1e-6 * np.abs(r[:, 8:11]) + 1e-9).all(), key
        nonzero += int((np.abs(r[:, 5:11]) > 0).any(axis=1).sum())
        if key == "mdr_37":
            for row in r:
                k1, v1 = find_pc(row[1] ** 2, row[2:5])
                assert np.abs(k1 - row[5:8]).max() <= 1e-8
                assert (np.abs(v1 - row[8:11]) <= 1e-6 * np.abs(row[8:11]) + 1e-9).all()
    assert nonzero > 400          # the candidates search is exercised, not only the empty case


def test_oracle_zone_flags_agree(sisi):
    """in_ws of the oracle and zone_flags of the package on random and
    boundary points of the primitive zone."""
    from phinfortran_gb300.unfold_pc import zone_flags
    rec = sisi_primitive_cell(sisi).recivec
    rng = np.random.default_rng(3)
    ks = np.concatenate([rng.uniform(-2, 2, (200, 3)), 0.5 * rec, 0.5 * (rec[0] + rec[1])[None]])
    assert (zone_flags(rec, ks) == np.array([U.in_ws(rec, k) for k in ks])).all()
    assert (zone_flags(rec, 0.5 * rec) == 2).all()


def test_read_primitive_cell_fdf(tmp_path, sisi):
    f = sisi
    text = ["NumberOfAtoms 4", "NumberOfSpecies 1", f"LatticeConstant {float(f['pc_lscale'])} Ang",
            "%block LatticeVectors"] + [" ".join(repr(float(x)) for x in v) for v in f["pc_latvec"]] + \
           ["%endblock LatticeVectors", "%block AtomicScaledCoordinatesAndAtomicSpecies"] + \
           [" ".join(repr(float(x)) for x in p) + f" {int(s)}" for p, s in zip(f["pc_scaled"], f["pc_species"])] + \
           ["%endblock AtomicScaledCoordinatesAndAtomicSpecies"]
    path = tmp_path / "pc.fdf"
    path.write_text("\n".join(text) + "\n")
    d = read_primitive_cell_fdf(str(path))
    assert np.array_equal(d["latvec"], f["pc_latvec"]) and np.array_equal(d["scaled"], f["pc_scaled"])
    assert np.array_equal(d["species"], f["pc_species"]) and d["lscale"] == float(f["pc_lscale"])


def test_write_mode_files_appends_in_order(tmp_path, perk):
    """The reference opens the files with POSITION='APPEND': two calls for
    the same k extend one file; names carry the 1-based k number."""
    rows = perk["left_0"]
    first = [tuple(r) for r in rows[:3]]
    second = [tuple(r) for r in rows[3:5]]
    write_mode_files(str(tmp_path), {"left": [(0, first)]})
    write_mode_files(str(tmp_path), {"left": [(0, second)], "mdl": [(4, [])]}, k_index={0: 1, 4: 12})
    path = tmp_path / "left_specular_param_000001.dat"
    back = np.loadtxt(path, ndmin=2)
    np.testing.assert_allclose(back, rows[:5], rtol=1e-9, atol=0)
    assert (tmp_path / "mdl_specular_param_000012.dat").exists()


def test_mode_rows_assembly_matches_oracle_rows(sisi):
    """modes.mode_rows (the host half of the per-k files) fed with per-mode
    data built from the oracle's matrices -- k_z, labels and the per-label
    column sums the GPU entry returns -- gives the oracle's rows exactly,
    mode order included."""
    from phinfortran_gb300.modes import KINDS, MATRICES, LeadGeometry, mode_rows

    f = sisi
    ik, ies = 37, [5, 11, 25, 50]
    nb = tuple(int(x) for x in f["n_bloch"])
    b, p = int(f["buffer"]), int(f["period"])
    geo = LeadGeometry.from_qe(f["pos_all"], f["cell"], f["cell_all"], nb, b, p, b, p)
    cell = f["cell"]
    reci_uc = 2 * np.pi * np.linalg.inv(cell).T
    geom = dict(ksc=f["kgrid"][ik], recivec=2 * np.pi * np.linalg.inv(f["cell_all"]).T, reci_uc_l=reci_uc,
                reci_uc_r=reci_uc, nb=nb)
    pts = oracle_point_sums(f, ik, ies)
    nl = pts[0][0]["rll"].shape[0]
    nr = pts[0][0]["rrr"].shape[0]
    mm, ns = max(nl, nr), nb[0] * nb[1]
    res = dict(mode_kz=np.zeros((len(ies), 4, mm)), mode_bz=np.zeros((len(ies), 4, mm), np.int32),
               col_sums=np.zeros((len(ies), 4, mm, ns)), nl=nl, nr=nr)
    rows_of = {"tlr": ("ret_l", "adv_r"), "trl": ("ret_r", "adv_l"), "rrr": ("ret_r", "adv_r"),
               "rll": ("ret_l", "adv_l")}
    for a, (o, _) in enumerate(pts):
        md = o["modes"]
        for ki, kind in enumerate(KINDS):
            m = md[kind]
            res["mode_kz"][a, ki, :m["kz"].size] = m["kz"]
            res["mode_bz"][a, ki, :m["bz"].size] = m["bz"]
        for mi, mat in enumerate(MATRICES):
            M2 = np.abs(o[mat]) ** 2
            br, bc = md[rows_of[mat][0]]["bz"], md[rows_of[mat][1]]["bz"]
            for c in range(M2.shape[1]):
                if bc[c] > 0:
                    for lab in range(1, ns + 1):
                        res["col_sums"][a, mi, c, lab - 1] = M2[br == lab, c].sum()
    E = f["E"][ies]
    got = mode_rows(res, geo, f["kgrid"][[ik]], E, pc=sisi_primitive_cell(f))
    find_pc = sisi_find_pc(f)
    for a, (o, _) in enumerate(pts):
        want = M.mode_file_rows(E[a], o, geom, find_pc)
        for name in FILES:
            g = np.array(got[name][a][1], dtype=np.float64).reshape(-1, 15 if name.startswith("md") else 14)
            w = np.array(want[name], dtype=np.float64).reshape(g.shape)
            np.testing.assert_allclose(g, w, rtol=1e-9, atol=1e-12, err_msg=f"{name} point {a}")


def test_mode_rows_from_oracle_modes_match_reference_files(sisi, perk):
    """The whole host half of the per-k files -- mode_rows on the per-mode
    data the GPU entry returns (here built from the oracle's matrices) with
    the package's primitive-cell unfolding -- against the reference's six
    files of k = 1, every energy and every column."""
    from phinfortran_gb300.modes import KINDS, MATRICES, LeadGeometry, mode_rows

    f, ik = sisi, 0
    nb = tuple(int(x) for x in f["n_bloch"])
    b, p = int(f["buffer"]), int(f["period"])
    geo = LeadGeometry.from_qe(f["pos_all"], f["cell"], f["cell_all"], nb, b, p, b, p)
    pts = oracle_point_sums(f, ik, list(range(f["E"].size)))
    nl, nr = pts[0][0]["rll"].shape[0], pts[0][0]["rrr"].shape[0]
    mm, ns = max(nl, nr), nb[0] * nb[1]
    res = dict(mode_kz=np.zeros((len(pts), 4, mm)), mode_bz=np.zeros((len(pts), 4, mm), np.int32),
               col_sums=np.zeros((len(pts), 4, mm, ns)), nl=nl, nr=nr)
    rows_of = {"tlr": ("ret_l", "adv_r"), "trl": ("ret_r", "adv_l"), "rrr": ("ret_r", "adv_r"),
               "rll": ("ret_l", "adv_l")}
    for a, (o, _) in enumerate(pts):
        md = o["modes"]
        for ki, kind in enumerate(KINDS):
            res["mode_kz"][a, ki, :md[kind]["kz"].size] = md[kind]["kz"]
            res["mode_bz"][a, ki, :md[kind]["bz"].size] = md[kind]["bz"]
        for mi, mat in enumerate(MATRICES):
            m2 = np.abs(o[mat]) ** 2
            br, bc = md[rows_of[mat][0]]["bz"], md[rows_of[mat][1]]["bz"]
            for c in np.nonzero(bc > 0)[0]:
                res["col_sums"][a, mi, c] = [m2[br == lab, c].sum() for lab in range(1, ns + 1)]
    rows = mode_rows(res, geo, f["kgrid"][[ik]], f["E"], pc=sisi_primitive_cell(f))
    for name in FILES:
        compare_rows([r for _, rr in rows[name] for r in rr], perk[f"{name}_{ik}"], name.startswith("md"))
