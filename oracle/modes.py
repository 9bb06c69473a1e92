"""Mode-resolved transmission of negf/velocity_mat.f90 (oracle; tests only).

Restates vel_mat_tdb (negf/velocity_mat.f90:1692-3148) for the quantities
it returns: the specular / non-specular split of the transmission and
reflection (transl_s, transl_ns, transr_s, transr_ns, refll_s, refll_ns,
reflr_s, reflr_ns), built from the Bloch eigenmodes of the four lead
transfer matrices, the velocity matrices, the t/r matrices
(velocity_mat.f90:2940-2963) and the supercell->primitive unfolding that
labels each propagating mode with a folded-BZ index (velocity_mat.f90:
2035-2126).  The path_mode != 1 branch is followed (Gram-Schmidt of the
propagating columns, no degenerate-state rotation).  The per-k text files
(write_specular / write_md) and the primitive-cell velocities of
find_k_pc feed only those files and are not restated.

Helpers restated from negf/util.f90: gram_schmidt (800-823, including its
conjugated projection coefficient), log_fbz (825-839), move_in_ws2
(675-706), sqrtm (359-454, Schur form + upper-triangular recurrence with
the zero-denominator guard).  The lead geometry setup is
transverse_uc_setup (velocity_mat.f90:14-179) in its qe_fc form
(negf/phinfortran.f90:122-160).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla

from . import negf as N

PI = 3.141592653589793238


def gram_schmidt(U1):
    """util.f90:800-823. coefficient = dot_product(U1_i, U2_j)/|U2_j|^2 with
    Fortran's dot_product (conjugates its first argument)."""
    U1 = np.asarray(U1, dtype=np.complex128)
    U2 = U1.copy()
    n = U1.shape[1]
    for i in range(1, n):
        for j in range(i):
            c = np.vdot(U1[:, i], U2[:, j]) / np.vdot(U2[:, j], U2[:, j])
            U2[:, i] = U2[:, i] - c * U2[:, j]
    for i in range(n):
        U2[:, i] = U2[:, i] / np.sqrt(np.vdot(U2[:, i], U2[:, i]))
    return U2


def log_fbz(lam, az):
    """util.f90:825-839: k_z folded into (-G/2, G/2]."""
    Gz = 2 * PI / az
    kz = np.real(np.log(lam) / (1j * az))
    kz = np.mod(kz, Gz)
    return kz - Gz if kz > Gz * 0.5 else kz


def move_in_ws2(k, a):
    """util.f90:675-706: the in-plane lattice translate of k closest to 0
    (first minimum over i1, i2 in -2..2, i1 outer)."""
    best, out = None, None
    for i1 in range(-2, 3):
        for i2 in range(-2, 3):
            d = k - (i1 * a[0] + i2 * a[1])
            dist = float(np.dot(d, d))
            if best is None or dist < best:
                best, out = dist, d
    return out


def sqrtm(A):
    """util.f90:359-454: complex Schur form A = Q S Q^H, U = sqrt(S) by the
    super-diagonal recurrence, U(i,j) = 0 where U(i,i) + U(j,j) == 0."""
    S, Q = sla.schur(np.asarray(A, dtype=np.complex128), output="complex")
    n = S.shape[0]
    U = np.zeros_like(S)
    for i in range(n):
        U[i, i] = np.sqrt(S[i, i])
    for sd in range(1, n):
        for i in range(n - sd):
            j = i + sd
            v = S[i, j] - np.dot(U[i, i + 1:j], U[i + 1:j, j])
            den = U[i, i] + U[j, j]
            U[i, j] = v / den if den != 0 else 0.0
    return Q @ U @ Q.conj().T


def lead_unfolding_setup(pos_all, cell_uc, n_bloch, buffer_left, period_left, buffer_right, period_right):
    """transverse_uc_setup (velocity_mat.f90:14-179) with positions = pos_all
    and latvec_uc = the QE cell.  Returns, per lead, the orbital positions
    (pos_l / pos_r), the representative atom of every orbital's transverse
    unit cell (pidx, 0-based into L_list) and L_list (0-based atom ids)."""
    pos_all = np.asarray(pos_all, dtype=np.float64)
    natoms = pos_all.shape[0]
    inv_uc = np.linalg.inv(cell_uc)
    nbx, nby = int(n_bloch[0]), int(n_bloch[1])

    def side(atoms, tol):
        lst = []
        for i in atoms:
            f = pos_all[i] @ inv_uc
            if -0.001 < f[0] < 0.999 and -0.001 < f[1] < 0.999:
                lst.append(i)
        pos, pidx = [], []
        temp = 0
        for i in atoms:
            p0 = pos_all[i]
            for j, a in enumerate(lst):
                for k in range(nbx):
                    for l in range(nby):
                        dp = p0 - pos_all[a] - (k * cell_uc[0] + l * cell_uc[1])
                        if np.sqrt(np.dot(dp, dp)) < tol:
                            temp = j
            for _ in range(3):
                pos.append(p0)
                pidx.append(temp)
        return dict(pos=np.array(pos), pidx=np.array(pidx, dtype=np.int64), list=np.array(lst, dtype=np.int64))

    left = side(range(buffer_left + period_left, buffer_left + 2 * period_left), 1.0e-3)
    right = side(range(natoms - buffer_right - 2 * period_right, natoms - buffer_right - period_right), 1.0e-5)
    return left, right


def unfold_weights(u, lam, ksc, recivec, reci_uc, lead, pos_all, nb):
    """Unfolding weights of one mode over the nb folded k shifts
    (velocity_mat.f90:2035-2072); returns (nb,) weights."""
    nbx, nby = nb
    nbt = nbx * nby
    n = u.shape[0]
    stride = n // nbt
    kc = ksc @ recivec
    w = np.zeros(nbt)
    natm = lead["list"].size
    shifts = [(i, j) for i in range(nbx) for j in range(nby)]
    for js, (sx, sy) in enumerate(shifts):
        kpoint = move_in_ws2((np.array([sx, sy, 0.0]) + ksc) @ recivec, reci_uc)
        t = 0
        for _ in range(natm):
            idx = lead["pidx"][t]
            pos_uc = pos_all[lead["list"][idx]]
            for it in range(3):
                rows = t + it + stride * np.arange(nbt)
                pos = lead["pos"][rows]
                ph = np.exp(-1j * (-(pos @ kc) + (pos - pos_uc) @ kpoint))
                s = np.sum(ph * u[rows] * lam)
                w[js] += abs(s) ** 2 / nbt
            t += 3
    return w


def _lead_modes(F, Gm, sign_v, use_inv_h, sign_kz, E, az, lambda_eta, ksc, recivec, reci_uc, lead, pos_all, nb):
    """Eigenmodes of one transfer matrix, the velocity matrix, its square
    root, the inverse used by the t/r matrices and the BZ labels."""
    lam, U = np.linalg.eig(F)
    n = F.shape[0]
    prop = np.nonzero(np.abs(np.abs(lam) - 1.0) < lambda_eta)[0]
    kz = np.full(n, 100.0)
    for i in prop:
        kz[i] = sign_kz * log_fbz(lam[i], az)
    if prop.size:
        U[:, prop] = gram_schmidt(U[:, prop])
    V = sign_v * (U.conj().T @ Gm @ U) * 1j * az / 2.0 / np.sqrt(E)
    Uinv = np.linalg.inv(U.conj().T) if use_inv_h else np.linalg.inv(U)
    Vh = sqrtm(V)
    bz = np.zeros(n, dtype=np.int64)
    for i in prop:
        w = unfold_weights(U[:, i], lam[i], ksc, recivec, reci_uc, lead, pos_all, nb)
        bz[i] = int(np.argmax(w)) + 1
    return dict(lam=lam, U=U, kz=kz, V=V, Vh=Vh, Uinv=Uinv, bz=bz, prop=prop)


def split_sums(M, bz_row, bz_col):
    """s / ns sums of |M_ij|^2 (velocity_mat.f90:3035-3106)."""
    a = np.abs(M) ** 2
    br = bz_row[:, None]
    bc = bz_col[None, :]
    s = np.sum(a[(br == bc) & (br > 0)])
    ns = np.sum(a[(br != bc) & (bc > 0) & (br > 0)])
    return float(s), float(ns)


def vel_mat_tdb(E, first, blocks, surf, rgf, geom, eta, eta0, lambda_eta):
    """One (E, k) point.  ``surf``: raw surface_green_tdb outputs for this
    point (gl_adv, gr_ret, gl_plus, gr_minus, gml_adv, gmr_ret); ``rgf``:
    G_D_RL, G_D_LR, G_L, G_R; ``geom``: dict(ksc, recivec, reci_uc_l,
    reci_uc_r, a_z_l, a_z_r, left, right, pos_all, nb).  Returns the eight
    sums and the t/r matrices."""
    H = N.H
    gl, gr = surf["gl_adv"], surf["gr_ret"]
    glp, grm = surf["gl_plus"], surf["gr_minus"]
    gml, gmr = surf["gml_adv"], surf["gmr_ret"]
    HL, HR, HLv, HRv = blocks["HL"], blocks["HR"], blocks["HLv"], blocks["HRv"]
    g = geom
    common = dict(E=E, lambda_eta=lambda_eta, ksc=g["ksc"], recivec=g["recivec"], pos_all=g["pos_all"], nb=g["nb"])
    aL = _lead_modes(gl @ HLv, gml, -1.0, True, -1.0, az=g["a_z_l"], reci_uc=g["reci_uc_l"], lead=g["left"], **common)
    rL = _lead_modes(H(gl) @ HLv, H(gml), -1.0, False, -1.0, az=g["a_z_l"], reci_uc=g["reci_uc_l"], lead=g["left"],
                     **common)
    rR = _lead_modes(gr @ HRv, gmr, 1.0, False, 1.0, az=g["a_z_r"], reci_uc=g["reci_uc_r"], lead=g["right"], **common)
    aR = _lead_modes(H(gr) @ HRv, H(gmr), 1.0, True, 1.0, az=g["a_z_r"], reci_uc=g["reci_uc_r"], lead=g["right"],
                     **common)
    eps = E * eta + eta0
    nl, nr = HL.shape[0], HR.shape[0]
    QL = (E + eps * 1j) * np.eye(nl) - HL - H(HLv) @ H(gl) @ HLv - HLv @ glp @ H(HLv)
    QR = (E + eps * 1j) * np.eye(nr) - HR - H(HRv) @ gr @ HRv - HRv @ H(grm) @ H(HRv)
    azl, azr = g["a_z_l"], g["a_z_r"]
    trl = 1j * (rR["Vh"] @ (rR["Uinv"] @ (rgf["G_D_RL"] @ (aL["Uinv"] @ aL["Vh"])))) * 2.0 * np.sqrt(E / azr / azl)
    tlr = 1j * (rL["Vh"] @ (rL["Uinv"] @ (rgf["G_D_LR"] @ (aR["Uinv"] @ aR["Vh"])))) * 2.0 * np.sqrt(E / azl / azr)
    rrr = 1j * (rR["Vh"] @ (rR["Uinv"] @ ((rgf["G_R"] - np.linalg.inv(QR)) @ (aR["Uinv"] @ aR["Vh"])))) * 2.0 * \
        np.sqrt(E / azr / azr)
    rll = 1j * (rL["Vh"] @ (rL["Uinv"] @ ((rgf["G_L"] - np.linalg.inv(QL)) @ (aL["Uinv"] @ aL["Vh"])))) * 2.0 * \
        np.sqrt(E / azl / azl)
    if first:
        trl = np.zeros_like(trl)
        tlr = np.zeros_like(tlr)
        rrr = np.zeros_like(rrr)
        rll = np.zeros_like(rll)
    out = {}
    # transr_* from trl (rows: right ret, cols: left adv), transl_* from tlr
    out["transr_s"], out["transr_ns"] = split_sums(trl, rR["bz"], aL["bz"])
    out["transl_s"], out["transl_ns"] = split_sums(tlr, rL["bz"], aR["bz"])
    out["reflr_s"], out["reflr_ns"] = split_sums(rrr, rR["bz"], aR["bz"])
    out["refll_s"], out["refll_ns"] = split_sums(rll, rL["bz"], aL["bz"])
    out.update(trl=trl, tlr=tlr, rrr=rrr, rll=rll, modes=dict(adv_l=aL, ret_l=rL, ret_r=rR, adv_r=aR))
    return out


def k_xyz(mode, ksc, recivec, reci_uc, nb):
    """velocity_mat.f90:2353-2360: the unfolded in-plane k of every
    propagating mode (its label's shift) with z = k_z; 100 elsewhere."""
    shifts = [(i, j) for i in range(nb[0]) for j in range(nb[1])]
    k = np.full((mode["kz"].size, 3), 100.0)
    for i in mode["prop"]:
        sx, sy = shifts[mode["bz"][i] - 1]
        k[i] = move_in_ws2((np.array([sx, sy, 0.0]) + ksc) @ recivec, reci_uc)
        k[i, 2] = mode["kz"][i]
    return k


def _spec_sums(r, kf, kb, i):
    """The r_s / r_t loop of negf/write_data.f90:39-57 for incoming mode i."""
    rt = rs = 0.0
    for j in range(kf.shape[0]):
        if kf[j, 2] < 99.9:
            a = abs(r[j, i]) ** 2
            rt += a
            d = kf[j] - kb[i]
            d[2] = 0.0
            if d @ d < 1.0e-5:
                rs += a
    rt = 1.0e-60 if 0.0 < rt < 1.0e-60 else rt
    rs = 1.0e-60 if 0.0 < rs < 1.0e-60 else rs
    return rs, rt


def write_specular_rows(w, r, kf, kb, pcb=None):
    """negf/write_data.f90:3-76; pcb (nb, 6): k_pc and v_pc of the incoming
    modes (zero when None)."""
    pcb = np.zeros((kb.shape[0], 6)) if pcb is None else pcb
    rows, c = [], 0
    for i in range(kb.shape[0]):
        if kb[i, 2] < 99.9:
            c += 1
            rs, rt = _spec_sums(r, kf, kb, i)
            rows.append((c, w, *kb[i], *pcb[i], rs, rt, rs / rt if rt != 0.0 else 0.0))
    return rows


def write_md_rows(w, t, r, kft, kf, kb, pcb=None):
    """negf/write_data.f90:78-176; pcb as in write_specular_rows."""
    pcb = np.zeros((kb.shape[0], 6)) if pcb is None else pcb
    rows, c = [], 0
    for i in range(kb.shape[0]):
        if kb[i, 2] < 99.9:
            c += 1
            rs, rt = _spec_sums(r, kf, kb, i)
            ts, tt = _spec_sums(t, kft, kb, i)
            rows.append((c, w, *kb[i], *pcb[i], rs, rt, ts, tt))
    return rows


def mode_file_rows(E, o, geom, find_pc=None):
    """Rows of the six per-k files for one point of vel_mat_tdb
    (velocity_mat.f90:3108-3128).  find_pc(E, k) -> (k_pc, v_pc) gives the
    primitive-cell columns (oracle/unfold_pc.find_k_pc; zero when None)."""
    g = geom
    md = o["modes"]
    kl = lambda m: k_xyz(m, g["ksc"], g["recivec"], g["reci_uc_l"], g["nb"])
    kr = lambda m: k_xyz(m, g["ksc"], g["recivec"], g["reci_uc_r"], g["nb"])
    kLr, kLa, kRr, kRa = kl(md["ret_l"]), kl(md["adv_l"]), kr(md["ret_r"]), kr(md["adv_r"])

    def pcols(kb):
        out = np.zeros((kb.shape[0], 6))
        if find_pc is not None:
            for i in range(kb.shape[0]):
                if kb[i, 2] < 99.9:
                    kp, vp = find_pc(E, kb[i])
                    out[i, :3], out[i, 3:] = kp, vp
        return out

    pLa, pRa = pcols(kLa), pcols(kRa)
    w = float(np.sqrt(E))
    return dict(tlr=write_specular_rows(w, o["tlr"], kLr, kRa, pRa),
                trl=write_specular_rows(w, o["trl"], kRr, kLa, pLa),
                right=write_specular_rows(w, o["rrr"], kRr, kRa, pRa),
                left=write_specular_rows(w, o["rll"], kLr, kLa, pLa),
                mdl=write_md_rows(w, o["trl"], o["rll"], kRr, kLr, kLa, pLa),
                mdr=write_md_rows(w, o["tlr"], o["rrr"], kLr, kRr, kRa, pRa))
