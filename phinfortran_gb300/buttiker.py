"""Buttiker probes (inelastic scattering) of the tdb branch over the C ABI.

With ``buttiker = 1`` the reference adds to every device layer i a probe
self-energy sigma_w(i, ie) (set_sigma_bp_w, negf/lesser.f90:12-45), solves
the probe-aware Green's function and the lesser function of every (k, E)
point (get_G_full_tdb / get_G_lesser_tdb, negf/lesser.f90:475-1503) and
updates the probe temperatures by a Newton step on the omega-integrated
probe fluxes until they carry no net heat (negf/phinfortran.f90:1157-1290,
negf/lesser.f90:1506-1623).  ``probe_points`` runs the per-point part on the
GPU (``pf_buttiker_tdb``); ``probe_loop`` is the host iteration around it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .transport import BLOCK_NAMES, TdbBlocks, fortran_block

PI = 3.141592653589793238     # negf/util.f90:5
KB = 1.380649e-23             # negf/util.f90:9
HBAR = 1.0545718e-34          # negf/util.f90:10


def bose_einstein(freq, T):
    """negf/util.f90:987-999, freq in THz."""
    x = np.exp(HBAR * freq * 1.0e12 * 2 * PI / KB / T)
    return 1.0 / (x - 1.0)


def dbosedT(freq, T):
    """negf/util.f90:1001-1013."""
    x = np.exp(HBAR * freq * 1.0e12 * 2 * PI / KB / T)
    return x / (x - 1.0) ** 2 * HBAR * freq * 1.0e12 * 2 * PI / KB / T ** 2


def simpson(x, y):
    """negf/util.f90:1015-1043 (uniform step x[-1] - x[-2], odd count)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y)
    n = x.size
    if (n - 1) % 2:
        raise ValueError("the number of energies must be odd (Simpson rule)")
    # the reference adds y1, the 4-weighted odd points, the 2-weighted even
    # points and y_n in that order
    f = y[0] + 0.0j
    f = f + np.sum(4.0 * y[1:n - 1:2])
    f = f + np.sum(2.0 * y[2:n - 1:2])
    f = f + y[n - 1]
    return f * (x[-1] - x[-2]) / 3.0


def initial_temperatures(nlayer, t_left, t_right):
    """negf/phinfortran.f90:187-199: linear profile over the middle half."""
    if nlayer > 1:
        i = np.arange(nlayer)
        return t_left + 0.25 * (t_right - t_left) + 0.5 * i * (t_right - t_left) / (nlayer - 1)
    return np.array([float(t_left)])


def sigma_probe(temps, Egrid, B_probe, T_probe, lifetime=1):
    """negf/lesser.f90:12-45: (sigma_w, dsigma_wdt), each (nlayer, ne)."""
    temps = np.asarray(temps, dtype=np.float64)[:, None]
    E = np.asarray(Egrid, dtype=np.float64)[None, :]
    tau = 1.0 / (B_probe * E * temps * np.exp(-T_probe / temps))
    sw = -2.0j * np.sqrt(E) / tau
    dsw = -2.0j * np.sqrt(E) * (B_probe * E * np.exp(-T_probe / temps) * (1.0 + T_probe / temps))
    if lifetime == 0:
        sw = np.zeros_like(sw)
    return sw, dsw


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def probe_points(E, blocks, sigw, dsigw, temps, t_left, t_right, *, eta, eta0, convergence, dev_factor=10.0,
                 qidx=None, first=None, max_iter=1000, check=True):
    """Per point: T_L, probe fluxes, lead fluxes, Tr A_i, Tr Gn_i and the
    Jacobian d flux_i / d T_j.  sigw, dsigw (npts, L) at each point's energy."""
    lib = _abi.load()
    if isinstance(blocks, dict):
        blocks = TdbBlocks.from_dict(blocks)
    nq, (n, nl, nr, L), arrs = blocks.stacked()
    buf = {k: fortran_block(v) for k, v in arrs.items()}
    E = np.ascontiguousarray(E, dtype=np.float64)
    npts = E.size
    freq = np.sqrt(E)
    temps = np.asarray(temps, dtype=np.float64)
    f = np.ascontiguousarray(np.stack([bose_einstein(freq, T) for T in temps], axis=1))
    df = np.ascontiguousarray(np.stack([dbosedT(freq, T) for T in temps], axis=1))
    fL = np.ascontiguousarray(bose_einstein(freq, t_left))
    fR = np.ascontiguousarray(bose_einstein(freq, t_right))
    sw = np.ascontiguousarray(np.asarray(sigw, dtype=np.complex128).reshape(npts, L))
    dsw = np.ascontiguousarray(np.asarray(dsigw, dtype=np.complex128).reshape(npts, L))
    q = None if qidx is None else np.ascontiguousarray(qidx, dtype=np.int32)
    fi = None if first is None else np.ascontiguousarray(first, dtype=np.int32)
    T = np.zeros(npts)
    flux = np.zeros((npts, L), np.complex128)
    jac = np.zeros((npts, L, L), np.complex128)
    A = np.zeros((npts, L), np.complex128)
    Gn = np.zeros((npts, L), np.complex128)
    fl = np.zeros(npts, np.complex128)
    fr = np.zeros(npts, np.complex128)
    st = np.zeros(npts, np.int32)
    v = lambda a: _p(a.view(np.float64))
    rc = lib.pf_buttiker_tdb(n, nl, nr, L, nq, *[_p(buf[k]) for k in BLOCK_NAMES], npts, _p(E),
                             None if q is None else _p(q, C.c_int), None if fi is None else _p(fi, C.c_int),
                             v(sw), v(dsw), _p(f), _p(df), _p(fL), _p(fR), eta, eta0, dev_factor, convergence,
                             max_iter, _p(T), v(flux), v(jac), v(A), v(Gn), v(fl), v(fr), _p(st, C.c_int))
    if rc != 0 and (check or rc != -4):
        raise _abi.PFError(rc, lib.pf_buttiker_last_error().decode(errors="replace"))
    return dict(transl=T, flux_i=flux, jacobian=jac, A_sum=A, Gn_i=Gn, flux_left=fl, flux_right=fr, status=st)


def probe_loop(Egrid, blocks_per_k, t_left, t_right, B_probe, T_probe, *, eta, eta0, convergence,
               dev_factor=10.0, lifetime=1, max_iter=100, tol=1.0e-4, temps=None):
    """Newton iteration on the probe temperatures (negf/phinfortran.f90:1157-1290).

    Egrid (ne,) odd; blocks_per_k: one tdb block set per k (equal weights).
    Each pass solves all (k, E) points on the GPU, integrates fluxes and
    Jacobian over omega (integrate_jacobian, negf/lesser.f90:1506-1529),
    steps T <- T - Re(J^-1 flux) (update_temperature, :1531-1557) and
    updates the probe self-energies; it stops when the rms change falls
    below tol.  Returns dict(temps, temps_ph, iterations, tdiff, transl)."""
    Egrid = np.asarray(Egrid, dtype=np.float64)
    ne = Egrid.size
    nk = len(blocks_per_k)
    L = np.asarray(blocks_per_k[0]["Hd"]).shape[0]
    temps = initial_temperatures(L, t_left, t_right) if temps is None else np.asarray(temps, dtype=np.float64)
    temps_ph = temps.copy()
    w = np.sqrt(Egrid)
    first = (np.arange(ne) == 0).astype(np.int32)
    it, tdiff = 0, np.inf
    TL = np.zeros((nk, ne))
    for it in range(1, max_iter + 1):
        sw, dsw = sigma_probe(temps, Egrid, B_probe, T_probe, lifetime)
        flux_all = np.zeros((nk, ne, L), np.complex128)
        jac_all = np.zeros((nk, ne, L, L), np.complex128)
        A_all = np.zeros((nk, ne, L), np.complex128)
        Gn_all = np.zeros_like(A_all)
        for k, b in enumerate(blocks_per_k):
            r = probe_points(Egrid, b, sw.T, dsw.T, temps, t_left, t_right, eta=eta, eta0=eta0,
                             convergence=convergence, dev_factor=dev_factor, first=first)
            flux_all[k], jac_all[k], A_all[k], Gn_all[k] = r["flux_i"], r["jacobian"], r["A_sum"], r["Gn_i"]
            TL[k] = r["transl"]
        flux = np.array([simpson(w, flux_all[:, :, i].sum(axis=0) * w / nk) for i in range(L)])
        J = np.array([[simpson(w, jac_all[:, :, i, j].sum(axis=0) * w / nk) for j in range(L)] for i in range(L)])
        temps_ph = lattice_temperatures(A_all.sum(axis=0), Gn_all.sum(axis=0), Egrid, temps_ph)
        old = temps
        temps = old - np.real(np.linalg.inv(J) @ flux)
        if temps.min() < 0.0:
            temps = np.ones_like(temps)
        tdiff = float(np.sqrt(np.dot(temps - old, temps - old) / L))
        if tdiff < tol:
            break
    return dict(temps=temps, temps_ph=temps_ph, iterations=it, tdiff=tdiff, transl=TL)


def lattice_temperatures(A_sum, Gn_sum, Egrid, temps_ph):
    """negf/lesser.f90:1588-1623: per layer, the temperature whose Bose
    occupation reproduces the layer's lesser function (Newton, to 1e-4)."""
    E = np.asarray(Egrid, dtype=np.float64)
    w = np.sqrt(E)
    T = np.array(temps_ph, dtype=np.float64)
    for nn in range(T.size):
        old = -100.0
        while abs(old - T[nn]) > 1.0e-4:
            old = T[nn]
            jd = np.real(simpson(w, -dbosedT(w, T[nn]) * E * A_sum[:, nn]))
            d = np.real(simpson(w, Gn_sum[:, nn] * E - bose_einstein(w, T[nn]) * E * A_sum[:, nn]))
            T[nn] = old - d / jd
    return T
