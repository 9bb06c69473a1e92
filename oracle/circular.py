"""Restatement of the block-circulant surface Green's function (oracle;
tests only): negf/circular.f90:9-105 (set_pmatrix, circular_g) with
negf/util.f90:732-799 (fourier_transform, decimation).

With ``circular_flag = 1`` the reference replaces each Lopez-Sancho
decimation of surface_green_tdb (negf/surface.f90:498-590) by
``circular_g``: the lead matrices of an n_bloch_y x n_bloch_x Bloch
supercell are block circulant, so a Fourier transform along y and then x
makes them block diagonal, each of the nb*nc small blocks is decimated on
its own (util's ``decimation``, which takes beta = alpha^H), and the result
is transformed back with the unitary matrices P1, P2.  Mathematically this
is the decimation of the full matrices; the reference notes a 1e-10
difference (negf/circular.f90:47-48).
"""
from __future__ import annotations

import numpy as np


def fourier_transform(H, n, nb, G, R):
    """negf/util.f90:732-756: block i = sum_j H(block row 1, block j) exp(i G.R (i-1)(j-1)/nb)."""
    na = n // nb
    out = np.zeros((n, n), dtype=np.complex128)
    gr = float(np.dot(np.asarray(G, float), np.asarray(R, float)))
    for i in range(nb):
        acc = np.zeros((na, na), dtype=np.complex128)
        for j in range(nb):
            acc = acc + H[0:na, j * na:(j + 1) * na] * np.exp(1j * gr * (i / nb) * j)
        out[i * na:(i + 1) * na, i * na:(i + 1) * na] = acc
    return out


def set_pmatrix(n, nb, G, R):
    """negf/circular.f90:9-38: P((i-1)na+k, (j-1)na+k) = exp(i G.R (j-1)(i-1)/nb)/sqrt(nb)."""
    na = n // nb
    gr = float(np.dot(np.asarray(G, float), np.asarray(R, float)))
    P = np.zeros((n, n), dtype=np.complex128)
    for i in range(nb):
        for j in range(nb):
            for k in range(na):
                P[i * na + k, j * na + k] = np.exp(1j * gr * (j / nb) * i) / np.sqrt(float(nb))
    return P, P.conj().T


def decimation(Es0, e1, alpha, convergence, max_iter=10000):
    """negf/util.f90:761-799 (beta = alpha^H regardless of the argument)."""
    e1 = e1.copy()
    es = e1.copy()
    beta = alpha.conj().T
    it = 0
    while np.max(np.abs(alpha)) > convergence and it < max_iter:
        ive = np.linalg.inv(Es0 - e1)
        ab = alpha @ ive @ beta
        e1 = e1 + ab + beta @ ive @ alpha
        es = es + ab
        alpha, beta = alpha @ ive @ alpha, beta @ ive @ beta
        it += 1
    return np.linalg.inv(Es0 - es)


def circular_g(Es0, e1, alpha, beta, convergence, n, nb, nc, G1, R1, G2, R2, P1=None, P2=None):
    """negf/circular.f90:42-105.  P1 (n) and P2 (n/nb) default to the
    matrices of (G1, R1) and (G2, R2); the reference builds both once from
    the left lead and uses them for every lead (negf/phinfortran.f90:622-628)."""
    na = n // nb
    nac = na // nc
    if P1 is None:
        P1 = set_pmatrix(n, nb, G1, R1)
    if P2 is None:
        P2 = set_pmatrix(na, nc, G2, R2)
    E0 = fourier_transform(Es0, n, nb, G1, R1)
    F1 = fourier_transform(e1, n, nb, G1, R1)
    A = fourier_transform(alpha, n, nb, G1, R1)
    green1 = np.zeros((n, n), dtype=np.complex128)
    for i in range(nb):
        s = slice(i * na, (i + 1) * na)
        Ey = fourier_transform(E0[s, s], na, nc, G2, R2)
        ey = fourier_transform(F1[s, s], na, nc, G2, R2)
        ay = fourier_transform(A[s, s], na, nc, G2, R2)
        green2 = np.zeros((na, na), dtype=np.complex128)
        for j in range(nc):
            t = slice(j * nac, (j + 1) * nac)
            green2[t, t] = decimation(Ey[t, t], ey[t, t], ay[t, t], convergence)
        green1[s, s] = P2[0] @ green2 @ P2[1]
    return P1[0] @ green1 @ P1[1]


def transport_circular(E, blocks, eta, eta0, convergence, dev_factor, n_bloch_y, n_bloch_x, gr,
                       zero_first=None):
    """T_L of one q with circular_flag = 1: surface_green_tdb's two decimations
    on the transmission path (left advanced, negf/surface.f90:479-507; right
    retarded, :540-568) through circular_g, then the wrapper conjugations
    (negf/lesser.f90:141-144) and the sweep and Caroli trace of
    get_G_full_tdb (oracle.negf.get_G_full_tdb).  ``gr``: the G.R products
    {left y, left x, right y, right x}; P1, P2 from the left lead's
    (negf/phinfortran.f90:622-628)."""
    from oracle import negf as N
    E = np.asarray(E, dtype=np.float64)
    HL, HLv, HR, HRv = (np.asarray(blocks[k], dtype=np.complex128) for k in ("HL", "HLv", "HR", "HRv"))
    n = HL.shape[0]
    ny, nx = int(n_bloch_y), int(n_bloch_x)
    ey, ex = np.array([1.0, 0.0, 0.0]), np.array([0.0, 1.0, 0.0])
    # G and R enter only through G.R: carry each product on unit vectors
    GRl = (gr[0] * ey, ey, gr[1] * ex, ex)
    GRr = (gr[2] * ey, ey, gr[3] * ex, ex)
    P1 = set_pmatrix(n, ny, GRl[0], GRl[1])
    P2 = set_pmatrix(n // ny, nx, GRl[2], GRl[3])
    eps = N.lead_eps(E, eta, eta0)
    B = E.size
    gl_adv = np.zeros((B, n, n), np.complex128)
    gr_ret = np.zeros((B, n, n), np.complex128)
    for b in range(B):
        zl, zr = E[b] - 1j * eps[b], E[b] + 1j * eps[b]
        a = N.H(HLv)
        gl_adv[b] = circular_g(zl * np.eye(n), HL, a, N.H(a), convergence, n, ny, nx, *GRl, P1=P1, P2=P2)
        a = N.H(HRv)
        gr_ret[b] = circular_g(zr * np.eye(n), HR, a, N.H(a), convergence, n, ny, nx, *GRr, P1=P1, P2=P2)
    sl_adv = N.H(HLv) @ gl_adv @ HLv
    gml_adv = 1j * (sl_adv - N.H(sl_adv))
    sr_ret = N.H(HRv) @ gr_ret @ HRv
    gmr_ret = 1j * (sr_ret - N.H(sr_ret))
    r = N.get_G_full_tdb(E, N.H(gl_adv), gr_ret, -gml_adv, gmr_ret, N.H(sl_adv), sr_ret,
                         blocks["Hd"], blocks["Hdv"], blocks["Hld"], blocks["Hrd"], HL, HR,
                         eta, eta0, dev_factor, zero_first=zero_first)
    return r["transl"]
