"""FP64 numpy restatement of the NEGF transport kernels (oracle; tests only).

Every array is complex128.  Matrices are stored as numpy (..., rows, cols)
arrays; batching is over a leading point axis B (one point = one energy at
one transverse q).  Each routine follows the reference step for step, only
vectorised over B.  Convergence is tracked per point exactly as the
reference's scalar ``do while`` does: a point stops iterating the moment its
own ``maxval(abs(alpha))`` drops to ``convergence``.

Energy model (unifies the phonon tdb branch and the electron tb branch):

* lead broadening     eps(E) = E*eta + eta0
    - phonon: negf/surface.f90:479,510,540,571 (``E*eta+eta0``)
    - tb:     tb/surface.f90:216 etc. use a fixed ``eta``; pass eta=0, eta0=eta
* device energy       z_D = E + i*dev_factor*eps(E)
    - phonon: dev_factor = 10 (negf/lesser.f90:556,581,615,705,731,757)
    - tb:     dev_factor = 1  (tb/device.f90:390,...)

Block naming (all column-major in the reference, row/col here):
    HL  = Haml   lead cell onsite                   (n_l x n_l)
    HLv = Hamlv  H_{-1,0}: outer left cell -> cell 0 (n_l x n_l)
    HR  = Hamr,  HRv = Hamrv = H_{N+2,N+1}           (n_r x n_r)
    Hd[i]  = Hamd(i)   device layer onsite           (n x n), i = 1..L
    Hdv[i] = Hamdv(i)  H_{i,i+1}                     (n x n), i = 1..L-1
    Hld = Hamld  H_{0,1}                             (n_l x n)
    Hrd = Hamrd  H_{N+1,N}                           (n_r x n)
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "H", "lead_eps", "decimate", "surface_green_tdb", "get_G_full_tdb",
    "transport", "T_CLAMP",
]

T_CLAMP = 1.0e-60   # negf/lesser.f90:795-800 and negf/write_data.f90:368-373


def H(a):
    """Conjugate transpose of the trailing two axes (Fortran transpose(dconjg()))."""
    return np.conj(np.swapaxes(a, -1, -2))


def lead_eps(E, eta, eta0):
    """Lead broadening E*eta+eta0 (negf/surface.f90:479)."""
    return np.asarray(E, dtype=np.float64) * eta + eta0


def _eye(n):
    return np.eye(n, dtype=np.complex128)


def decimate(zs, H00, alpha, beta, convergence, max_iter=None):
    """Lopez-Sancho decimation, batched over points.

    Follows negf/surface.f90:488-497 (identical loop at :518-526, :548-557,
    :579-588 and tb/surface.f90:216-232 ...):

        ive   = inv(Es0 - e1)
        e1    = e1 + alpha ive beta + beta ive alpha
        es    = es + alpha ive beta
        alpha = alpha ive alpha
        beta  = beta ive beta
        until maxval(|alpha|) <= convergence;   g = inv(Es0 - es)

    ``zs``: (B,) complex energies; ``H00``/``alpha``/``beta``: (n,n) or (B,n,n).
    Returns (g (B,n,n), iterations (B,) int).  ``max_iter=None`` reproduces
    the reference's unbounded loop.
    """
    zs = np.asarray(zs, dtype=np.complex128)
    B = zs.shape[0]
    n = H00.shape[-1]
    e1 = np.broadcast_to(H00, (B, n, n)).astype(np.complex128).copy()
    es = e1.copy()
    al = np.broadcast_to(alpha, (B, n, n)).astype(np.complex128).copy()
    be = np.broadcast_to(beta, (B, n, n)).astype(np.complex128).copy()
    Es0 = zs[:, None, None] * _eye(n)
    iters = np.zeros(B, dtype=np.int64)
    active = np.abs(al).reshape(B, -1).max(axis=1) > convergence
    while active.any():
        idx = np.nonzero(active)[0]
        if max_iter is not None:
            idx = idx[iters[idx] < max_iter]
            if idx.size == 0:
                break
        ive = np.linalg.inv(Es0[idx] - e1[idx])
        a, b = al[idx], be[idx]
        a_ive = a @ ive
        b_ive = b @ ive
        aib = a_ive @ b
        e1[idx] = e1[idx] + aib + b_ive @ a
        es[idx] = es[idx] + aib
        al[idx] = a_ive @ a
        be[idx] = b_ive @ b
        iters[idx] += 1
        active[:] = False
        active[idx] = np.abs(al[idx]).reshape(idx.size, -1).max(axis=1) > convergence
    g = np.linalg.inv(Es0 - es)
    return g, iters


def surface_green_tdb(E, HL, HLv, HR, HRv, eta, eta0, convergence,
                      max_iter=None, want_plus_minus=True):
    """Four lead decimations of negf/surface.f90:385-605 (tb: tb/surface.f90:129-343).

    Returns a dict with gl_adv, gl_plus, gr_ret, gr_minus, sl_adv, sr_ret,
    gml_adv, gmr_ret (each (B,n,n)) and the iteration counts.
    """
    E = np.asarray(E, dtype=np.float64)
    eps = lead_eps(E, eta, eta0)
    out = {}
    # left, advanced (surface.f90:479-507)
    gl_adv, it_la = decimate(E - 1j * eps, HL, H(HLv), HLv, convergence, max_iter)
    sl_adv = H(HLv) @ gl_adv @ HLv
    gml_adv = 1j * (sl_adv - H(sl_adv))
    out.update(gl_adv=gl_adv, sl_adv=sl_adv, gml_adv=gml_adv, it_l_adv=it_la)
    if want_plus_minus:
        # left, reflected (surface.f90:510-532)
        gl_plus, it_lp = decimate(E + 1j * eps, HL, HLv, H(HLv), convergence, max_iter)
        out.update(gl_plus=gl_plus, it_l_plus=it_lp)
    # right, retarded (surface.f90:540-568)
    gr_ret, it_rr = decimate(E + 1j * eps, HR, H(HRv), HRv, convergence, max_iter)
    sr_ret = H(HRv) @ gr_ret @ HRv
    gmr_ret = 1j * (sr_ret - H(sr_ret))
    out.update(gr_ret=gr_ret, sr_ret=sr_ret, gmr_ret=gmr_ret, it_r_ret=it_rr)
    if want_plus_minus:
        # right, reflected (surface.f90:571-593)
        gr_minus, it_rm = decimate(E - 1j * eps, HR, HRv, H(HRv), convergence, max_iter)
        out.update(gr_minus=gr_minus, it_r_minus=it_rm)
    return out


def get_G_full_tdb(E, gl, gr, gml, gmr, sl, sr, Hd, Hdv, Hld, Hrd, HL, HR,
                   eta, eta0, dev_factor, zero_first=None, want_blocks=False):
    """Both RGF sweeps and the Caroli traces of negf/lesser.f90:475-809.

    The arguments are what get_G_full_tdb receives from its wrapper
    (negf/lesser.f90:141-149): ``gl`` = gl_adv^H (retarded), ``gml`` = -gml_adv,
    ``sl`` = sl_adv^H, ``gr``/``gmr``/``sr`` the right retarded quantities.
    The electron G_block (tb/device.f90:291-575) is the same recursion with
    dev_factor=1.  Only the quantities on the transmission path are formed;
    the backward G_full/G_q_qp pass (lesser.f90:661-680) feeds the lesser
    function, which is outside this path.

    ``zero_first``: boolean (B,) mask of points forced to T=0 (the reference's
    ``ie == 1`` rule, lesser.f90:802-807).  Values below 1e-60 become 0
    (lesser.f90:795-800).
    """
    E = np.asarray(E, dtype=np.float64)
    B = E.shape[0]
    L = Hd.shape[0]
    n = Hd.shape[-1]
    zD = E + 1j * dev_factor * lead_eps(E, eta, eta0)
    In = _eye(n)
    Es = zD[:, None, None] * In
    # ---- left-to-right sweep (lesser.f90:547-609) ----
    V = Hld
    g = np.linalg.inv(Es - Hd[0] - H(V) @ gl @ V)
    G0N = gl @ V @ g
    for i in range(1, L):
        V = Hdv[i - 1]
        g = np.linalg.inv(Es - Hd[i] - H(V) @ g @ V)
        G0N = G0N @ V @ g
    # right lead block (lesser.f90:613-654)
    nr = HR.shape[-1]
    EsR = zD[:, None, None] * _eye(nr)
    GRinv = EsR - HR - sr
    V = H(Hrd)                                   # (n, n_r)
    GRR = np.linalg.inv(GRinv - H(V) @ g @ V)    # G_{N+1,N+1}
    G_D_LR = G0N @ V @ GRR                       # G_{0,N+1}
    # ---- right-to-left sweep (lesser.f90:694-784) ----
    V = Hrd                                      # (n_r, n)
    g = np.linalg.inv(Es - Hd[L - 1] - H(V) @ gr @ V)
    GNo = gr @ V @ g
    for i in range(L - 1, 0, -1):
        V = H(Hdv[i - 1])
        g = np.linalg.inv(Es - Hd[i - 1] - H(V) @ g @ V)
        GNo = GNo @ V @ g
    nl = HL.shape[-1]
    EsL = zD[:, None, None] * _eye(nl)
    GLinv = EsL - HL - sl
    V = Hld                                      # (n_l, n)
    GLL = np.linalg.inv(GLinv - V @ g @ H(V))    # G_{0,0}
    G_D_RL = GNo @ H(V) @ GLL                    # G_{N+1,0}
    # ---- Caroli (lesser.f90:787-800) ----
    GGGGl = (G_D_LR @ gmr) @ (H(G_D_LR) @ gml)
    GGGGr = (G_D_RL @ gml) @ (H(G_D_RL) @ gmr)
    transl = np.real(np.trace(GGGGl, axis1=-2, axis2=-1)).copy()
    transr = np.real(np.trace(GGGGr, axis1=-2, axis2=-1)).copy()
    transl[transl < T_CLAMP] = 0.0
    transr[transr < T_CLAMP] = 0.0
    if zero_first is not None:
        zf = np.asarray(zero_first, dtype=bool)
        transl[zf] = 0.0
        transr[zf] = 0.0
    out = dict(transl=transl, transr=transr)
    if want_blocks:
        out.update(G_D_LR=G_D_LR, G_D_RL=G_D_RL, G_R=GRR, G_L=GLL)
    return out


def transport(E, blocks, eta, eta0, convergence, dev_factor, zero_first=None,
              max_iter=None, want_blocks=False, want_plus_minus=False):
    """Surface decimation + both sweeps + Caroli for one q and a batch of E.

    ``blocks``: dict with HL, HLv, HR, HRv, Hd (L,n,n), Hdv (L-1,n,n), Hld, Hrd.
    This is the per-(ie,ik) body of negf/phinfortran.f90:1196-1213
    (surface_green_tdb_mpi then get_G_full_tdb_mpi) batched over ie.
    """
    s = surface_green_tdb(E, blocks["HL"], blocks["HLv"], blocks["HR"], blocks["HRv"],
                          eta, eta0, convergence, max_iter=max_iter,
                          want_plus_minus=want_plus_minus)
    # wrapper conjugations, negf/lesser.f90:141-144
    gl = H(s["gl_adv"])
    gml = -s["gml_adv"]
    sl = H(s["sl_adv"])
    r = get_G_full_tdb(E, gl, s["gr_ret"], gml, s["gmr_ret"], sl, s["sr_ret"],
                       blocks["Hd"], blocks["Hdv"], blocks["Hld"], blocks["Hrd"],
                       blocks["HL"], blocks["HR"], eta, eta0, dev_factor,
                       zero_first=zero_first, want_blocks=want_blocks)
    r["iters_left"] = s["it_l_adv"]
    r["iters_right"] = s["it_r_ret"]
    r["surface"] = s
    return r
