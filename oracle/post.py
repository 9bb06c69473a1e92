"""Post-processing restatements (oracle; tests only).

``condt`` -- two-probe Landauer conductance of examples/negf/si-si/condt.py:14-30:
    sigma(T) = 1/A * 1/(2 pi) * trapz( hbar w * df/dT * T(w), w ),
    f = 1/(exp(hbar w / kB T) - 1),  w in rad/s.
``kavg_from_files`` -- the k-average condt.py applies (sum of the nk columns / nk,
condt.py:44-51) and the omega conversion sqrt(E) * 2 pi 1e12 (condt.py:51).
"""
from __future__ import annotations

import numpy as np

KB = 1.380649e-23          # condt.py:10
HBAR = 1.0545718e-34       # condt.py:11
THZ2RADS = 1e12 * np.pi * 2  # condt.py:12


def condt(w, T, trans, area):
    """condt.py:14-30 (np.trapz over w)."""
    w = np.asarray(w, dtype=np.float64)
    trans = np.asarray(trans, dtype=np.float64)
    expf = np.exp(HBAR * w / KB / T)
    dfdw = expf / (expf - 1) ** 2 * HBAR * w / KB / T ** 2
    itd = 1 / area / 2 / np.pi * (HBAR * w * dfdw * trans)
    return float(np.sum((itd[1:] + itd[:-1]) * 0.5 * np.diff(w)))


def omega_from_egrid(E):
    """condt.py:51: omega = sqrt(E) * 2 pi 1e12 (E in THz^2)."""
    return np.sqrt(np.asarray(E, dtype=np.float64)) * THZ2RADS
