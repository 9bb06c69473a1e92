"""The reference's transmission output files (negf/write_data.f90:340-497).

``write_trans`` writes the ten tables the phonon driver produces at the end
of a run -- transl_s/ns, refll_s/ns, transr_s/ns, reflr_s/ns, transl_tot,
transr_tot -- in the same text format: one row per energy, the energy then
one column per k, every number in Fortran ``1e24.16`` edit format, values
below 1e-60 written as zero (negf/write_data.f90:364-370 etc.).  The left
tables and the reflection tables end each row with a blank (``" "``), the
right and total tables with nothing, as the reference's WRITE statements do.
"""
from __future__ import annotations

import os

import numpy as np

CLAMP = 1.0e-60


def fortran_e(x, w=24, d=16):
    """One value in Fortran Ew.d edit format (0.ddd...E+xx, right-justified).

    Exponents beyond two digits drop the 'E' as the standard prescribes
    (0.dddd-100)."""
    x = float(x)
    if x == 0.0 or not np.isfinite(x):
        if x == 0.0:
            body = "0." + "0" * d + "E+00"
        else:
            body = "NaN" if x != x else ("Infinity" if x > 0 else "-Infinity")
        return body.rjust(w)
    sign = "-" if x < 0 else ""
    s = f"{abs(x):.{d - 1}e}"                   # d significant digits, correctly rounded
    mant, ex = s.split("e")
    digits = mant.replace(".", "")
    e10 = int(ex) + 1                           # 0.ddd form
    if abs(e10) <= 99:
        tail = f"E{'+' if e10 >= 0 else '-'}{abs(e10):02d}"
    else:
        tail = f"{'+' if e10 >= 0 else '-'}{abs(e10):03d}"
    out = f"{sign}0.{digits}{tail}"
    if len(out) > w:
        return "*" * w
    return out.rjust(w)


def _table(path, E, T, end):
    T = np.array(T, dtype=np.float64, copy=True)
    T[T < CLAMP] = 0.0
    with open(path, "w") as f:
        for i in range(T.shape[0]):
            f.write(fortran_e(E[i]))
            f.write("".join(fortran_e(v) for v in T[i]))
            f.write(end + "\n")


def write_trans(output_dir, E, transl, transr, transl_s=None, transl_ns=None, transr_s=None, transr_ns=None,
                refll_s=None, refll_ns=None, reflr_s=None, reflr_ns=None):
    """Write the reference's transmission tables into output_dir.

    E: (ne,) energy grid (the reference writes E(i, 1), the grid of the
    first k); every table (ne, nk).  Tables given as None are not written
    (a T-only run writes transl_tot and transr_tot)."""
    os.makedirs(output_dir, exist_ok=True)
    E = np.asarray(E, dtype=np.float64).reshape(-1)
    blank = [("transl_s", transl_s, " "), ("transl_ns", transl_ns, " "), ("refll_s", refll_s, " "),
             ("refll_ns", refll_ns, " "), ("transr_s", transr_s, ""), ("transr_ns", transr_ns, ""),
             ("reflr_s", reflr_s, ""), ("reflr_ns", reflr_ns, ""), ("transl_tot", transl, ""),
             ("transr_tot", transr, "")]
    written = []
    for name, T, end in blank:
        if T is None:
            continue
        T = np.asarray(T, dtype=np.float64)
        if T.ndim == 1:
            T = T[:, None]
        if T.shape[0] != E.size:
            raise ValueError(f"{name}: {T.shape[0]} rows for {E.size} energies")
        p = os.path.join(output_dir, name + ".dat")
        _table(p, E, T, end)
        written.append(p)
    return written


def read_table(path):
    """(E, T) of a table written by the reference or by write_trans."""
    a = np.loadtxt(path, ndmin=2)
    return a[:, 0], a[:, 1:]


def mode_file_line(row):
    """One row of a per-k mode file: count in I5, then the values in
    Fortran E20.10 (formats 1000 of negf/write_data.f90:69 and :171)."""
    return f"{int(row[0]):5d}" + "".join(fortran_e(v, 20, 10) for v in row[1:]) + "\n"


def write_mode_files(output_dir, rows, k_index=None):
    """Append the per-k mode files ``{name}_specular_param_{k:06d}.dat``
    (negf/write_data.f90:3-176) for the rows of ``modes.mode_rows``.

    ``rows``: {name: [(q, rows)] in point order}; ``k_index`` maps q to the
    reference's 1-based k number (default q + 1).  Like the reference the
    files are opened for appending, so points are written in the order
    given (energy order for one k) and an existing file grows."""
    os.makedirs(output_dir, exist_ok=True)
    for name, per_point in rows.items():
        files = {}
        try:
            for q, rr in per_point:
                k = (k_index[q] if k_index is not None else q + 1)
                if k not in files:
                    files[k] = open(os.path.join(output_dir, f"{name}_specular_param_{int(k):06d}.dat"), "a")
                files[k].writelines(mode_file_line(r) for r in rr)
        finally:
            for f in files.values():
                f.close()


def md2md_line(row):
    """One row of a mode-to-mode file: format 1000 of write_md2md
    (negf/write_data.f90:239), (2I5, 21E20.10, 2I5)."""
    c1, c2, *vals = row
    i, j = vals[-2:]
    return (f"{int(c1):5d}{int(c2):5d}" + "".join(fortran_e(v, 20, 10) for v in vals[:-2]) +
            f"{int(i):5d}{int(j):5d}\n")


def write_md2md_files(output_dir, rows, k_index=None):
    """Append the mode-to-mode files ``{direction}_md2md_{k:06d}.dat``
    (write_md2md, negf/write_data.f90:177-241, written by vel_mat_tdb with
    verbosity = 1, velocity_mat.f90:3132-3145) for the rows of
    ``modes.md2md_rows``; ``k_index`` maps q to the 1-based k number."""
    os.makedirs(output_dir, exist_ok=True)
    for direction, per_point in rows.items():
        files = {}
        try:
            for q, rr in per_point:
                k = (k_index[q] if k_index is not None else q + 1)
                if k not in files:
                    files[k] = open(os.path.join(output_dir, f"{direction}_md2md_{int(k):06d}.dat"), "a")
                files[k].writelines(md2md_line(r) for r in rr)
        finally:
            for f in files.values():
                f.close()
