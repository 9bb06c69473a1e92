"""Shared helpers: rebuild the si-si tdb blocks from the golden fixture."""
from __future__ import annotations

import numpy as np

from oracle import dyn as D


def qe_from_fixture(f):
    return dict(fc=f["fc"], cell=f["cell"], pos=f["pos"], mass=f["mass"], nx=int(f["nxyz"][0]),
                ny=int(f["nxyz"][1]), nz=int(f["nxyz"][2]), cell_sc=f["cell_sc"], rws=f["rws"], rd=f["rd"])


def sisi_blocks(f, ik):
    """tdb blocks of k point ik (0-based) through the oracle's dyn.f90 restatement."""
    qe = qe_from_fixture(f)
    nb = f["n_bloch"]
    return D.gen_dyn_qe_tdb_k(f["kgrid"][ik], qe, f["cell_all"], f["pos_all"], f["idxall"], f["mass_all"],
                              int(nb[0]), int(nb[1]), int(f["nz"]), int(f["buffer"]), int(f["period"]),
                              int(f["buffer"]), int(f["period"]), int(f["nlayer"]), int(f["natm_layer"]))


def sisi_params(f):
    return dict(eta=float(f["eta"]), eta0=float(f["eta0"]), convergence=float(f["convergence"]),
                dev_factor=float(f["dev_factor"]))


def golden_close(T, G, abs_tol=1e-6, rel_q99=1e-8):
    """Parity rule against the reference's committed FP64 output.

    The si-si run uses eta = 1e-8, so a few (omega, k) points are
    ill-conditioned: there the reference's own T_L and T_R differ by up to
    1.25e-7.  The rule is: every point within abs_tol (1e-6 absolute on
    T ~ 1..16), and 99% of points with T > 1e-3 within rel_q99 relative.
    """
    T = np.asarray(T)
    G = np.asarray(G)
    ad = np.abs(T - G)
    big = np.abs(G) > 1e-3
    rel = ad[big] / np.abs(G[big])
    q99 = np.quantile(rel, 0.99) if rel.size else 0.0
    return bool(ad.max() <= abs_tol and q99 <= rel_q99), float(ad.max()), float(q99)


def fp64_noise_floor(E, blocks, params, trials=3, rel=1e-15, seed=11):
    """Per-point FP64 conditioning of T: max |dT| of the oracle over `trials`
    random relative perturbations of size `rel` (about 5 ulp) of every block.

    Two correct FP64 implementations that round differently can disagree by
    this much; near subband edges with eta = 1e-6 it reaches ~1e-8.
    """
    from oracle import negf as N
    rng = np.random.default_rng(seed)
    base = N.transport(E, blocks, params["eta"], params["eta0"], params["convergence"],
                       params["dev_factor"])
    dev = np.zeros(len(E))
    for _ in range(trials):
        bp = {}
        for k, v in blocks.items():
            v = np.asarray(v, dtype=np.complex128)
            bp[k] = v * (1 + rel * rng.standard_normal(v.shape))
        o = N.transport(E, bp, params["eta"], params["eta0"], params["convergence"], params["dev_factor"])
        dev = np.maximum(dev, np.abs(o["transl"] - base["transl"]))
    return base, dev


def sisi_qe(f):
    """The processed QE force constants of the fixture as the primitive-cell
    unfolding takes them."""
    return dict(pos=f["pos"], cell=f["cell"], fc=f["fc"], rws=f["rws"], rd=f["rd"], nxyz=f["nxyz"])


def sisi_primitive_cell(f):
    """unfold_pc.PrimitiveCell of the si-si leads (pc1.fdf on both sides)."""
    from phinfortran_gb300.unfold_pc import PrimitiveCell
    nb = f["n_bloch"]
    return PrimitiveCell(sisi_qe(f), f["pc_latvec"], f["pc_scaled"], f["pc_species"], float(f["pc_lscale"]),
                         f["mass_no"], 2 * np.pi * np.linalg.inv(f["cell"]).T, int(max(nb[0], nb[1])))


def sisi_find_pc(f):
    """The oracle's find_k_pc for the si-si leads, as find_pc(E, k)."""
    from oracle import unfold_pc as U
    pos_pc, rec_pc, mass_uc = U.primitive_cell(f["pc_latvec"], f["pc_scaled"], f["pc_species"],
                                               float(f["pc_lscale"]), f["mass_no"])
    dyn = U.PcDyn(sisi_qe(f), pos_pc.shape[0], mass_uc)
    reci_uc = 2 * np.pi * np.linalg.inv(f["cell"]).T
    nb = f["n_bloch"]
    return lambda E, k: U.find_k_pc(E, k, reci_uc, rec_pc, dyn, int(max(nb[0], nb[1])))
