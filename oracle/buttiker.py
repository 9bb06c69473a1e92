"""Restatement of the Buttiker-probe (inelastic) path of the tdb branch
(oracle; tests only).

* ``set_sigma_bp_w``     -- negf/lesser.f90:12-45 (probe self-energy per layer
                            and energy, and its temperature derivative)
* ``bose_einstein``, ``dbosedT``, ``simpson`` -- negf/util.f90:987-1044
* ``initial_temperatures`` -- negf/phinfortran.f90:187-199
* ``g_full_probes``      -- negf/lesser.f90:475-680 (get_G_full_tdb with the
                            probe self-energies: the left-connected blocks
                            GLeft, the diagonal blocks G_full, the
                            off-diagonal G_q_qp, and T_L)
* ``g_lesser``           -- negf/lesser.f90:1199-1503 (get_G_lesser_tdb: the
                            left-connected and full lesser functions, their
                            temperature derivatives, probe fluxes, the
                            Jacobian, the lead fluxes)
* ``integrate_jacobian``, ``update_temperature``, ``get_ph_temperature`` --
                            negf/lesser.f90:1506-1623
* ``probe_loop``         -- the Newton iteration of negf/phinfortran.f90:1157-1290

Arrays are batched over points (leading axis B).  Matrices are numpy
(rows, cols); layers are uniform (the tdb branch), 0-based.
"""
from __future__ import annotations

import numpy as np

from .negf import H, lead_eps, surface_green_tdb

PI = 3.141592653589793238     # negf/util.f90:5
KB = 1.380649e-23             # negf/util.f90:9
HBAR = 1.0545718e-34          # negf/util.f90:10


def bose_einstein(freq, T):
    """negf/util.f90:987-999 (freq in THz)."""
    x = np.exp(HBAR * freq * 1.0e12 * 2 * PI / KB / T)
    return 1.0 / (x - 1.0)


def dbosedT(freq, T):
    """negf/util.f90:1001-1013."""
    x = np.exp(HBAR * freq * 1.0e12 * 2 * PI / KB / T)
    return x / (x - 1.0) ** 2 * HBAR * freq * 1.0e12 * 2 * PI / KB / T ** 2


def simpson(x, y):
    """negf/util.f90:1015-1043: composite Simpson with dx = x[-1] - x[-2]."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y)
    n = x.size
    if (n - 1) % 2:
        raise ValueError("ne should be an odd number")
    dx = x[-1] - x[-2]
    mm = (n - 1) // 2
    f = y[0] + 0.0j
    for i in range(1, mm + 1):
        f = f + 4.0 * y[2 * i - 1]
    for i in range(1, mm):
        f = f + 2.0 * y[2 * i]
    f = f + y[n - 1]
    return f * dx / 3.0


def initial_temperatures(nlayer, t_left, t_right):
    """negf/phinfortran.f90:187-199."""
    if nlayer > 1:
        i = np.arange(nlayer)
        return t_left + 0.25 * (t_right - t_left) + 0.5 * i * (t_right - t_left) / (nlayer - 1)
    return np.array([float(t_left)])


def set_sigma_bp_w(temps, Egrid, B_probe, T_probe, lifetime=1):
    """negf/lesser.f90:12-45: sigma_w[j, ie] = -2 i sqrt(E)/tau, tau = 1/(B E T exp(-C/T)),
    and dsigma_wdt = -2 i sqrt(E) B E exp(-C/T) (1 + C/T).  lifetime = 0 zeroes
    sigma_w (not its derivative), as the reference does."""
    temps = np.asarray(temps, dtype=np.float64)
    E = np.asarray(Egrid, dtype=np.float64)
    sw = np.zeros((temps.size, E.size), dtype=np.complex128)
    dsw = np.zeros_like(sw)
    for j, T in enumerate(temps):
        tau = 1.0 / (B_probe * E * T * np.exp(-T_probe / T))
        sw[j] = -2.0j * np.sqrt(E) / tau
        dsw[j] = -2.0j * np.sqrt(E) * (B_probe * E * np.exp(-T_probe / T) * (1.0 + T_probe / T))
    if lifetime == 0:
        sw[:] = 0.0
    return sw, dsw


def g_full_probes(E, gl, gr, gml, gmr, sr, Hd, Hdv, Hld, Hrd, HR, sigw, eta, eta0, dev_factor):
    """negf/lesser.f90:475-680 for a batch of points (one q).

    gl/gml/gr/gmr/sr are what get_G_full_tdb receives (gl = gl_adv^H, gml =
    -gml_adv); sigw (B, L) the probe self-energy of every layer.  Returns
    dict(GLeft (B, L, n, n), G_full (B, L, n, n), G_q_qp (B, L-1, n, n),
    transl (B,)).  As in the reference, GLeft[L-1] is replaced by the block
    closed with the right lead (Gblock_NN1) and G_full[L-1] equals it."""
    E = np.asarray(E, dtype=np.float64)
    L, n = Hd.shape[0], Hd.shape[-1]
    if L < 2:
        raise ValueError("the probe recursion needs at least two layers")
    zD = E + 1j * dev_factor * lead_eps(E, eta, eta0)
    Es = zD[:, None, None] * np.eye(n)
    I = np.eye(n)
    GLeft = np.zeros((E.size, L, n, n), np.complex128)
    V = Hld
    g = np.linalg.inv(Es - Hd[0] - H(V) @ gl @ V - sigw[:, 0, None, None] * I)
    GLeft[:, 0] = g
    G0N = gl @ V @ g
    NN1 = None
    for i in range(1, L):
        V = Hdv[i - 1]
        base = Es - Hd[i] - H(V) @ g @ V - sigw[:, i, None, None] * I
        gn = np.linalg.inv(base)
        if i == L - 1:
            V1 = H(Hrd)
            NN1 = np.linalg.inv(base - V1 @ gr @ H(V1))
        GLeft[:, i] = gn
        G0N = G0N @ V @ gn
        g = gn
    nr = HR.shape[-1]
    GRinv = zD[:, None, None] * np.eye(nr) - HR - sr
    V = H(Hrd)
    GRR = np.linalg.inv(GRinv - H(V) @ g @ V)
    G_D_LR = G0N @ V @ GRR
    T = np.real(np.trace(G_D_LR @ gmr @ H(G_D_LR) @ gml, axis1=-2, axis2=-1))
    T = np.where(T < 1.0e-60, 0.0, T)
    GLeft[:, L - 1] = NN1
    G_full = np.zeros_like(GLeft)
    G_full[:, L - 1] = NN1
    G_q_qp = np.zeros((E.size, L - 1, n, n), np.complex128)
    for i in range(L - 2, -1, -1):
        V = Hdv[i]
        qpq = G_full[:, i + 1] @ H(V) @ GLeft[:, i]
        G_q_qp[:, i] = GLeft[:, i] @ V @ G_full[:, i + 1]
        G_full[:, i] = GLeft[:, i] + GLeft[:, i] @ V @ qpq
    return dict(GLeft=GLeft, G_full=G_full, G_q_qp=G_q_qp, transl=T)


def _tr(a):
    return np.trace(a, axis1=-2, axis2=-1)


def g_lesser(E, first, gl, gr, GLeft, G_full, G_q_qp, Hdv, Hld, Hrd, sigw, dsigw, temps, t_left, t_right):
    """negf/lesser.f90:1199-1503 for a batch of points (one q).

    first: (B,) bool, the reference's ie == 1 (zero-frequency) points;
    sigw, dsigw: (B, L) probe self-energy and derivative at each point's
    energy; temps: (L,) probe temperatures.  Returns dict(flux_i (B, L),
    jacobian (B, L, L), A_sum (B, L), Gn_i (B, L), flux_left (B,),
    flux_right (B,)), all complex as in the reference."""
    E = np.asarray(E, dtype=np.float64)
    B, L, n = GLeft.shape[0], GLeft.shape[1], GLeft.shape[-1]
    I = np.eye(n)
    freq = np.sqrt(E)
    temps = np.asarray(temps, dtype=np.float64)
    f = np.stack([bose_einstein(freq, T) for T in temps], axis=1)        # (B, L)
    df = np.stack([dbosedT(freq, T) for T in temps], axis=1)
    fL = bose_einstein(freq, t_left)
    fR = bose_einstein(freq, t_right)
    # probe escape rates i (sigma - sigma^H), a multiple of the identity
    gi = 1j * (sigw - np.conj(sigw))          # (B, L)
    dgi = 1j * (dsigw - np.conj(dsigw))
    A = 1j * (G_full - H(G_full))
    s1 = H(Hld) @ gl @ Hld
    gamma_first = 1j * (s1 - H(s1))
    flux_left = _tr(gamma_first @ A[:, 0]) * fL
    GnL = np.zeros_like(GLeft)
    dGnL = np.zeros((B, L, L, n, n), np.complex128)          # dGnL[:, i, j] = dGnL_i / dT_j
    sig_in0 = gamma_first * fL[:, None, None] + gi[:, 0, None, None] * I * f[:, 0, None, None]
    GnL[:, 0] = GLeft[:, 0] @ sig_in0 @ H(GLeft[:, 0])
    dsig = gi[:, 0, None, None] * I * df[:, 0, None, None] + dgi[:, 0, None, None] * I * f[:, 0, None, None]
    dGnL[:, 0, 0] = GLeft[:, 0] @ dsig @ H(GLeft[:, 0])
    for i in range(1, L - 1):
        V = Hdv[i - 1]
        sig_prev = H(V) @ GnL[:, i - 1] @ V
        sig_in = gi[:, i, None, None] * I * f[:, i, None, None]
        Gi = GLeft[:, i]
        GnL[:, i] = Gi @ (sig_in + sig_prev) @ H(Gi)
        for j in range(i):
            dGnL[:, i, j] = Gi @ (H(V) @ dGnL[:, i - 1, j] @ V) @ H(Gi)
        dsig = gi[:, i, None, None] * I * df[:, i, None, None] + dgi[:, i, None, None] * I * f[:, i, None, None]
        dGnL[:, i, i] = Gi @ dsig @ H(Gi)
    # last layer, closed with the right lead
    V = Hdv[L - 2]
    sig_prev = H(V) @ GnL[:, L - 2] @ V
    V1 = H(Hrd)
    s_last = V1 @ gr @ H(V1)
    gamma_last = 1j * (s_last - H(s_last))
    flux_right = _tr(gamma_last @ A[:, L - 1]) * fR
    sig_in = gi[:, L - 1, None, None] * I * f[:, L - 1, None, None] + gamma_last * fR[:, None, None]
    Gi = GLeft[:, L - 1]
    GnL[:, L - 1] = Gi @ (sig_in + sig_prev) @ H(Gi)
    for j in range(L - 1):
        dGnL[:, L - 1, j] = Gi @ (H(V) @ dGnL[:, L - 2, j] @ V) @ H(Gi)
    dsig = (gi[:, L - 1, None, None] * I * df[:, L - 1, None, None]
            + dgi[:, L - 1, None, None] * I * f[:, L - 1, None, None])
    dGnL[:, L - 1, L - 1] = Gi @ dsig @ H(Gi)
    # full lesser function, right to left
    Gn = np.zeros_like(GnL)
    dGn = np.zeros_like(dGnL)
    Gn[:, L - 1] = GnL[:, L - 1]
    flux_right = (flux_right - _tr(gamma_last @ Gn[:, L - 1])) * freq
    dGn[:, L - 1] = dGnL[:, L - 1]
    for i in range(L - 2, -1, -1):
        V = Hdv[i]
        Gi = GLeft[:, i]
        Q = G_q_qp[:, i]
        Gn[:, i] = (GnL[:, i] + Gi @ V @ Gn[:, i + 1] @ H(V) @ H(Gi)
                    + GnL[:, i] @ V @ H(Q) + Q @ H(V) @ GnL[:, i])
        for j in range(L):
            X = dGnL[:, i, j]
            dGn[:, i, j] = X + Gi @ V @ dGn[:, i + 1, j] @ H(V) @ H(Gi) + X @ V @ H(Q) + Q @ H(V) @ X
    flux_left = (flux_left - _tr(gamma_first @ Gn[:, 0])) * freq
    z = np.asarray(first, dtype=bool)
    Gn[z] = 0.0
    dGn[z] = 0.0
    A[z] = 0.0
    trGn = _tr(Gn)                      # (B, L)
    trA = _tr(A)
    flux_i = -gi * trGn + gi * trA * f
    jac = -gi[:, :, None] * _tr(dGn)    # (B, L, L): -tr(gamma_i dGn_i/dT_j)
    idx = np.arange(L)
    jac[:, idx, idx] += gi * trA * df + dgi * trA * f
    return dict(flux_i=flux_i, jacobian=jac, A_sum=trA, Gn_i=trGn, flux_left=flux_left, flux_right=flux_right)


def integrate_jacobian(jac_all, flux_all, Egrid, nk):
    """negf/lesser.f90:1506-1529.  jac_all (nk, ne, L, L), flux_all (nk, ne, L)."""
    w = np.sqrt(np.asarray(Egrid, dtype=np.float64))
    L = flux_all.shape[-1]
    flux = np.zeros(L, np.complex128)
    J = np.zeros((L, L), np.complex128)
    for i in range(L):
        flux[i] = simpson(w, flux_all[:, :, i].sum(axis=0) * w / nk)
        for j in range(L):
            J[i, j] = simpson(w, jac_all[:, :, i, j].sum(axis=0) * w / nk)
    return J, flux


def update_temperature(J, flux, temps):
    """negf/lesser.f90:1531-1557: Newton step; a negative temperature resets
    all of them to 1.  Returns (new temps, tdiff)."""
    old = np.asarray(temps, dtype=np.float64)
    new = old - np.real(np.linalg.inv(J) @ flux)
    if new.min() < 0.0:
        new = np.ones_like(new)
    return new, float(np.sqrt(np.dot(new - old, new - old) / old.size))


def get_ph_temperature(A_sum, Gn_sum, Egrid, temps_ph):
    """negf/lesser.f90:1588-1623: per layer, the lattice temperature whose
    Bose occupation reproduces the local lesser function (Newton).
    A_sum, Gn_sum (ne, L) summed over k."""
    E = np.asarray(Egrid, dtype=np.float64)
    w = np.sqrt(E)
    T = np.array(temps_ph, dtype=np.float64)
    for nn in range(T.size):
        old = -100.0
        while abs(old - T[nn]) > 1.0e-4:
            old = T[nn]
            dfl = dbosedT(w, T[nn])
            fl = bose_einstein(w, T[nn])
            jd = np.real(simpson(w, -dfl * E * A_sum[:, nn]))
            d = np.real(simpson(w, Gn_sum[:, nn] * E - fl * E * A_sum[:, nn]))
            T[nn] = old - d / jd
    return T


def probe_point_batch(E, first, blocks, sigw, dsigw, temps, t_left, t_right, eta, eta0, convergence,
                      dev_factor=10.0):
    """One q: leads, probe-aware G and the lesser quantities for every point
    (the loop body of negf/phinfortran.f90:1196-1236 with buttiker = 1)."""
    s = surface_green_tdb(E, blocks["HL"], blocks["HLv"], blocks["HR"], blocks["HRv"], eta, eta0, convergence,
                          want_plus_minus=False)
    gl, gml, sr = H(s["gl_adv"]), -s["gml_adv"], s["sr_ret"]
    g = g_full_probes(E, gl, s["gr_ret"], gml, s["gmr_ret"], sr, blocks["Hd"], blocks["Hdv"], blocks["Hld"],
                      blocks["Hrd"], blocks["HR"], sigw, eta, eta0, dev_factor)
    r = g_lesser(E, first, gl, s["gr_ret"], g["GLeft"], g["G_full"], g["G_q_qp"], blocks["Hdv"], blocks["Hld"],
                 blocks["Hrd"], sigw, dsigw, temps, t_left, t_right)
    # get_G_full_tdb's ie == 1 rule (negf/lesser.f90:802-807)
    r["transl"] = np.where(np.asarray(first, dtype=bool), 0.0, g["transl"])
    return r


def probe_loop(Egrid, blocks_per_k, t_left, t_right, B_probe, T_probe, eta, eta0, convergence, dev_factor=10.0,
               lifetime=1, max_iter=100, tol=1.0e-4):
    """The Newton iteration of negf/phinfortran.f90:1157-1290 (buttiker = 1):
    every pass solves all (k, E) points at the current probe temperatures,
    integrates fluxes and Jacobian over omega (Simpson), takes one Newton
    step, updates the probe self-energies, and stops when the rms change is
    below tol.  Returns dict(temps, temps_ph, iterations, tdiff, transl)."""
    Egrid = np.asarray(Egrid, dtype=np.float64)
    L = blocks_per_k[0]["Hd"].shape[0]
    temps = initial_temperatures(L, t_left, t_right)
    temps_ph = temps.copy()
    nk = len(blocks_per_k)
    first = np.arange(Egrid.size) == 0
    tdiff = np.inf
    it = 0
    for it in range(1, max_iter + 1):
        sw, dsw = set_sigma_bp_w(temps, Egrid, B_probe, T_probe, lifetime)
        flux_all = np.zeros((nk, Egrid.size, L), np.complex128)
        jac_all = np.zeros((nk, Egrid.size, L, L), np.complex128)
        A_all = np.zeros_like(flux_all)
        Gn_all = np.zeros_like(flux_all)
        TL = np.zeros((nk, Egrid.size))
        for k, b in enumerate(blocks_per_k):
            r = probe_point_batch(Egrid, first, b, sw.T, dsw.T, temps, t_left, t_right, eta, eta0, convergence,
                                  dev_factor)
            flux_all[k], jac_all[k], A_all[k], Gn_all[k] = r["flux_i"], r["jacobian"], r["A_sum"], r["Gn_i"]
            TL[k] = r["transl"]
        J, flux = integrate_jacobian(jac_all, flux_all, Egrid, nk)
        temps_ph = get_ph_temperature(A_all.sum(axis=0), Gn_all.sum(axis=0), Egrid, temps_ph)
        temps, tdiff = update_temperature(J, flux, temps)
        if tdiff < tol:
            break
    return dict(temps=temps, temps_ph=temps_ph, iterations=it, tdiff=tdiff, transl=TL)
