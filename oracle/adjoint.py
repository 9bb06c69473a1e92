"""Adjoint (reverse-mode) derivative of the Caroli transmission (oracle; tests only).

There is no gradient in the reference; this is the FP64 reference gradient
the GPU adjoint is checked against (together with central finite
differences).  Notation of the extended block-tridiagonal matrix A over the
layers j = 0 (left lead cell), 1..L (device), L+1 (right lead cell), whose
left-connected recursion is the one of negf/lesser.f90:547-654:

    A_00 = gl^{-1},  A_jj = z_D - Hd_j,  A_{L+1} = z_D - HR - Sigma_R,
    A_{j,j+1} = -V_j,  V_0 = Hld, V_j = Hdv_j, V_L = Hrd^H.

T = Re Tr[X_0 Gamma_R X_0^H Gamma_L] with X = A^{-1} E_{L+1} (so X_0 is
G_{0,N+1}).  With W = Gamma_R X_0^H Gamma_L and G_{0,j} the block row 0 of
A^{-1}, a perturbation of the device blocks gives

    dT = Re Tr[dHd_j M_Hd_j] + Re Tr[dV_j M_V_j],
    M_Hd_j = 2 X_j W G_{0,j},
    M_V_j  = 2 (X_{j+1} W G_{0,j} + (X_j W G_{0,j+1})^H).

The lead blocks (and so the decimation) are held fixed: the derivative is
with respect to the device region and its couplings to the leads.
"""
from __future__ import annotations

import numpy as np

from . import negf as N

H = N.H


def transport_and_sensitivities(E, blocks, eta, eta0, convergence, dev_factor):
    """Return (T (B,), M dict) with M['Hd'] (B,L,n,n), M['Hdv'] (B,L-1,n,n),
    M['Hld'] (B,n,nl) for dHld (nl x n), M['Hrd'] (B,n,nr) for dHrd (nr x n)."""
    E = np.asarray(E, dtype=np.float64)
    s = N.surface_green_tdb(E, blocks["HL"], blocks["HLv"], blocks["HR"], blocks["HRv"], eta, eta0,
                            convergence, want_plus_minus=False)
    gl = H(s["gl_adv"])
    gml = -s["gml_adv"]
    gr = s["gr_ret"]
    gmr = s["gmr_ret"]
    sr = s["sr_ret"]
    Hd, Hdv, Hld, Hrd, HR = blocks["Hd"], blocks["Hdv"], blocks["Hld"], blocks["Hrd"], blocks["HR"]
    L = Hd.shape[0]
    zD = E + 1j * dev_factor * N.lead_eps(E, eta, eta0)
    B = E.size

    def V(j):
        if j == 0:
            return np.broadcast_to(Hld, (B,) + Hld.shape)
        if j == L:
            return np.broadcast_to(H(Hrd), (B,) + Hrd.shape[::-1])
        return np.broadcast_to(Hdv[j - 1], (B,) + Hdv.shape[1:])

    def Ajj(j):
        n = Hd.shape[-1]
        if j <= L:
            return zD[:, None, None] * np.eye(n) - Hd[j - 1]
        return zD[:, None, None] * np.eye(HR.shape[-1]) - HR - sr

    # block LU (left-connected factors), g_0 = gl
    g = [gl]
    for j in range(1, L + 2):
        Vp = V(j - 1)
        g.append(np.linalg.inv(Ajj(j) - H(Vp) @ g[j - 1] @ Vp))
    # X = A^{-1} E_{L+1}
    X = [None] * (L + 2)
    X[L + 1] = g[L + 1]
    for j in range(L, -1, -1):
        X[j] = g[j] @ V(j) @ X[j + 1]
    T = np.real(np.trace((X[0] @ gmr) @ (H(X[0]) @ gml), axis1=-2, axis2=-1))
    # row 0 of A^{-1}: solve A^H Z = E_0 with the factors g_j^H
    nl = gl.shape[-1]
    y = [None] * (L + 2)
    y[0] = H(g[0]) @ np.broadcast_to(np.eye(nl), gl.shape)
    for j in range(1, L + 2):
        y[j] = H(g[j]) @ H(V(j - 1)) @ y[j - 1]
    Z = [None] * (L + 2)
    Z[L + 1] = y[L + 1]
    for j in range(L, -1, -1):
        Z[j] = y[j] + H(g[j]) @ V(j) @ Z[j + 1]
    G0 = [H(z) for z in Z]          # G_{0,j}
    W = gmr @ H(X[0]) @ gml
    K = [X[j] @ W for j in range(L + 2)]
    M = dict(Hd=np.stack([2 * K[j] @ G0[j] for j in range(1, L + 1)], axis=1))
    MV = [2 * (K[j + 1] @ G0[j] + H(K[j] @ G0[j + 1])) for j in range(L + 1)]
    M["Hld"] = MV[0]
    M["Hrd"] = H(MV[L])                  # V_L = Hrd^H
    M["Hdv"] = (np.stack(MV[1:L], axis=1) if L > 1
                else np.zeros((B, 0) + Hd.shape[1:], dtype=np.complex128))
    return T, M


def directional_derivative(M, dblocks):
    """sum_blocks Re Tr[dB M_B] for a block perturbation dblocks (no batch axis)."""
    out = 0.0
    for k in ("Hd", "Hdv", "Hld", "Hrd"):
        if k in dblocks and np.size(dblocks[k]):
            d = np.asarray(dblocks[k])
            sub = "ij,bji->b" if d.ndim == 2 else "lij,blji->b"
            out = out + np.real(np.einsum(sub, d, M[k]))
    return out
