"""Output writer (phinfortran_gb300/output.py) against the reference's own
tables: the first rows of the ten si-si tables (tests/golden/
sisi_output_head.txt, verbatim from examples/negf/si-si/output) are parsed
and written again; the text must come back byte for byte.  Plus the Fortran
Ew.d edge cases and the 1e-60 clamp."""
import os

import numpy as np

from phinfortran_gb300 import output as W

HERE = os.path.dirname(os.path.abspath(__file__))


def heads():
    out, name = {}, None
    with open(os.path.join(HERE, "golden", "sisi_output_head.txt")) as f:
        for line in f:
            if line.startswith("# "):
                name = line[2:].strip()
                out[name] = []
            else:
                out[name].append(line)
    return out


def test_write_trans_reproduces_reference_text(tmp_path):
    h = heads()
    assert len(h) == 10
    tables = {}
    E = None
    for name, rows in h.items():
        a = np.array([[float(v) for v in r.split()] for r in rows])
        E = a[:, 0]
        tables[name] = a[:, 1:]
    W.write_trans(str(tmp_path), E, tables["transl_tot"], tables["transr_tot"],
                  **{k: v for k, v in tables.items() if k not in ("transl_tot", "transr_tot")})
    for name, rows in h.items():
        with open(tmp_path / (name + ".dat")) as f:
            mine = f.readlines()
        assert mine == rows, name


def test_fortran_e_format():
    assert W.fortran_e(0.0) == "  0.0000000000000000E+00"
    assert W.fortran_e(1.0e-6) == "  0.1000000000000000E-05"
    assert W.fortran_e(-2.5) == " -0.2500000000000000E+01"
    assert W.fortran_e(9.99999999999999999) == "  0.1000000000000000E+02"
    assert W.fortran_e(1.5e-120) == "  0.1500000000000000-119"
    assert len(W.fortran_e(123.456)) == 24


def test_clamp_and_row_endings(tmp_path):
    E = np.array([1.0, 2.0])
    T = np.array([[1e-70, 0.5], [2.0, -1.0]])     # < 1e-60 (negative too) is written as zero
    W.write_trans(str(tmp_path), E, T, T, transl_s=T)
    tot = open(tmp_path / "transl_tot.dat").read().splitlines()
    assert tot[0] == W.fortran_e(1.0) + W.fortran_e(0.0) + W.fortran_e(0.5)
    assert tot[1].endswith(W.fortran_e(0.0))
    s = open(tmp_path / "transl_s.dat").read().splitlines()
    assert s[0].endswith(" ") and not tot[0].endswith(" ")


def test_md2md_line_format():
    """write_md2md's format 1000 (negf/write_data.f90:239): 2I5, 21E20.10, 2I5."""
    from phinfortran_gb300.output import md2md_line
    row = (3, 1, 2.5, *([0.125] * 18), 0.25, 0.0, 2, 1)
    s = md2md_line(row)
    assert s.endswith("\n") and len(s) == 5 * 2 + 20 * 21 + 5 * 2 + 1
    assert s.startswith("    3    1") and s.rstrip("\n").endswith("    2    1")
    vals = s[10:10 + 20 * 21]
    assert vals[:20] == "    0.2500000000E+01"
    assert vals[20 * 19:20 * 20] == "    0.2500000000E+00" and vals[20 * 20:] == "    0.0000000000E+00"
