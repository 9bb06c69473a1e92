"""Run one benchmark workload through the engine and print a JSON summary.

    python -m phinfortran_gb300.run ribbon   --energies 64 --precision mixed
    python -m phinfortran_gb300.run diamond  --nc 3 --layers 4 --kpoints 2 --energies 8
    python -m phinfortran_gb300.run diamond  --nc 3 --layers 10 --energies 96 --circular --precision tc
    python -m phinfortran_gb300.run ribbon3  --width 256 --layers 1000 --energies 4 --perturb 1e-15
    python -m phinfortran_gb300.run sc       --layers 40 --energies 64 --mode grad --arith df64
    python -m phinfortran_gb300.run sisi     --kpoints 1 --energies 16 --mode modes
    python -m phinfortran_gb300.run sisi     --kpoints 49 --energies 61 --mode modes --out out/
    python -m phinfortran_gb300.run sisi     --kpoints 3 --energies 61 --mode modes --out out/ --md2md

Modes: ``transport`` (T per point), ``modes`` (T plus the s/ns sums of the
mode-resolved transmission; si-si fixture only), ``grad`` (adjoint: T and
the block sensitivities of the Landauer conductance).  ``--perturb r``
multiplies every block entry by (1 + r N(0,1)) first: two runs with and
without it give the FP64 conditioning of each point.  The summary gives
the wall time, the mean decimation count, the status words and T.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import systems as S


def _build(a):
    if a.workload == "ribbon":
        b, E, p = S.tb_ribbon(W=a.width or 32, L=a.layers or 200, ne=1024)
        return b, E[np.linspace(0, E.size - 1, a.energies).astype(int)], p, None
    if a.workload == "ribbon3":
        b, E, p = S.tb_ribbon3(W=a.width or 256, L=a.layers or 1000,
                               energies=np.linspace(700, 3300, a.energies).astype(int))
        return b, E, p, None
    if a.workload == "sc":
        b, E, p, aux = S.sc_phonon(nx=4, ny=4, L=a.layers or 40, ne=1024, mass_range=(1.0, 3.0),
                                   bond_range=(0.8, 1.2), seed_index=4)
        sel = np.linspace(1, E.size - 1, a.energies).astype(int)
        return b, E[sel], p, dict(aux, sel=sel)
    if a.workload == "diamond":
        kp = list(range(0, 64, max(1, 64 // a.kpoints)))[:a.kpoints]
        if a.gamma or a.circular:
            # the transverse Gamma point (block-circulant leads), one block set
            kp = [0]
            b, E, p, aux = S.diamond_phonon(nc=a.nc, L=a.layers or 60, nk_side=1)
        else:
            b, E, p, aux = S.diamond_phonon(nc=a.nc, L=a.layers or 60, kpoints=kp)
        Es = E[np.linspace(10, 500, a.energies).astype(int)]
        q = np.repeat(np.arange(len(kp), dtype=np.int32), Es.size)
        return b, np.tile(Es, len(kp)), p, dict(qidx=q)
    if a.workload == "sisi":
        return None
    raise SystemExit(f"unknown workload {a.workload}")


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("workload", choices=["ribbon", "ribbon3", "sc", "diamond", "sisi"])
    ap.add_argument("--mode", default="transport", choices=["transport", "modes", "grad"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "tc", "df64"])
    ap.add_argument("--arith", default="df64", choices=["fp64", "df64"], help="adjoint arithmetic")
    ap.add_argument("--ckpt", type=int, default=0, help="adjoint checkpoint interval (0: sqrt(L+2))")
    ap.add_argument("--energies", type=int, default=16)
    ap.add_argument("--kpoints", type=int, default=1)
    ap.add_argument("--layers", type=int, default=0)
    ap.add_argument("--width", type=int, default=0)
    ap.add_argument("--nc", type=int, default=2)
    ap.add_argument("--perturb", type=float, default=0.0)
    ap.add_argument("--gamma", action="store_true", help="diamond: the transverse Gamma point only")
    ap.add_argument("--circular", action="store_true",
                    help="diamond at the transverse Gamma point with the block-circulant lead option "
                         "(circular_flag = 1, nc x nc Bloch cells)")
    ap.add_argument("--out", default="",
                    help="sisi: write the reference's ten output tables and the per-k mode files into this directory")
    ap.add_argument("--md2md", action="store_true",
                    help="sisi with --out: also the mode-to-mode files (the reference's verbosity = 1)")
    a = ap.parse_args()
    import torch
    out = dict(workload=a.workload, mode=a.mode)
    if a.workload == "sisi":
        from .modes import LeadGeometry, transport_tdb_modes
        here = os.path.dirname(os.path.abspath(__file__))
        f = np.load(os.path.join(os.path.dirname(here), "tests", "golden", "sisi.npz"))
        from .dyn import gen_dyn_qe_tdb
        ks = list(range(0, 49, max(1, 49 // a.kpoints)))[:a.kpoints]
        buf, per = int(f["buffer"]), int(f["period"])
        blocks = gen_dyn_qe_tdb(f["kgrid"][ks], fc=f["fc"], cell=f["cell"], pos=f["pos"], cell_all=f["cell_all"],
                                pos_all=f["pos_all"], idxall=f["idxall"], mass_all=f["mass_all"], rws=f["rws"],
                                rd=f["rd"], n_bloch_x=int(f["n_bloch"][0]), n_bloch_y=int(f["n_bloch"][1]),
                                buffer_left=buf, period_left=per, buffer_right=buf, period_right=per,
                                nlayer=int(f["nlayer"]), natm_layer=int(f["natm_layer"]))
        if a.energies >= f["E"].size:
            E1 = f["E"]                         # the full grid; T of ie = 1 is zero (reference rule)
        else:
            E1 = f["E"][np.linspace(1, 60, a.energies).astype(int)]
        E = np.tile(E1, len(ks))
        zf = np.tile((np.arange(E1.size) == 0) & (E1.size == f["E"].size), len(ks)).astype(np.int32)
        q = np.repeat(np.arange(len(ks), dtype=np.int32), E1.size)
        p = dict(eta=float(f["eta"]), eta0=float(f["eta0"]), convergence=float(f["convergence"]),
                 dev_factor=float(f["dev_factor"]))
        nb = tuple(int(x) for x in f["n_bloch"])
        geo = LeadGeometry.from_qe(f["pos_all"], f["cell"], f["cell_all"], nb, buf, per, buf, per)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = transport_tdb_modes(E, blocks, geo, f["kgrid"][ks], qidx=q, zero_flag=zf, lambda_eta=5e-3,
                                a_z_l=f["cell"][2, 2], a_z_r=f["cell"][2, 2], check=False,
                                per_mode=bool(a.out), md2md=bool(a.out) and a.md2md, **p)
        torch.cuda.synchronize()
        out.update(points=int(E.size), seconds=time.perf_counter() - t0, transl=r["transl"].tolist(),
                   transl_s=r["transl_s"].tolist(), status=int(np.bitwise_or.reduce(r["status"])))
        if a.out:
            from .modes import SUM_NAMES, mode_rows
            from .output import write_mode_files, write_trans
            grid = lambda v: np.asarray(v).reshape(len(ks), E1.size).T      # (ne, nk) as the reference
            write_trans(a.out, E1, grid(r["transl"]), grid(r["transr"]), **{k: grid(r[k]) for k in SUM_NAMES})
            # the per-k mode files, numbered by the k's place in the 49-point grid,
            # with the primitive-cell columns of pc1.fdf (both leads)
            from .unfold_pc import PrimitiveCell
            qe = dict(pos=f["pos"], cell=f["cell"], fc=f["fc"], rws=f["rws"], rd=f["rd"], nxyz=f["nxyz"])
            pc = PrimitiveCell(qe, f["pc_latvec"], f["pc_scaled"], f["pc_species"], float(f["pc_lscale"]),
                               f["mass_no"], 2 * np.pi * np.linalg.inv(f["cell"]).T, max(nb))
            write_mode_files(a.out, mode_rows(r, geo, f["kgrid"][ks], E, qidx=q, pc=pc),
                             k_index={i: k + 1 for i, k in enumerate(ks)})
            if a.md2md:
                from .modes import md2md_rows
                from .output import write_md2md_files
                write_md2md_files(a.out, md2md_rows(r, geo, f["kgrid"][ks], E, qidx=q, pc=pc),
                                  k_index={i: k + 1 for i, k in enumerate(ks)})
            out["written"] = a.out
        print(json.dumps(out))
        return
    b, E, p, aux = _build(a)
    if a.perturb:
        rng = np.random.default_rng(7)
        b = {k: np.asarray(v) * (1 + a.perturb * rng.standard_normal(np.shape(v))) for k, v in b.items()}
    qidx = aux.get("qidx") if aux else None
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if a.mode == "grad":
        from .gradients import landauer_weights, transport_grad
        w = landauer_weights(aux["omega"][aux["sel"]], 300.0)
        T, M, st = transport_grad(E, b, w, ckpt=a.ckpt, arith=a.arith, check=False, **p)
        torch.cuda.synchronize()
        out.update(points=int(E.size), seconds=time.perf_counter() - t0, transl=T.tolist(),
                   status=int(np.bitwise_or.reduce(st)))
    else:
        from .transport import transport_tdb
        circ = (a.nc, a.nc, [2.0 * np.pi] * 4) if (a.circular and a.workload == "diamond") else None
        r = transport_tdb(E, b, qidx=qidx, want_transr=False, check=False, precision=a.precision, circular=circ,
                          **p)
        torch.cuda.synchronize()
        out.update(points=int(E.size), seconds=time.perf_counter() - t0, transl=r["transl"].tolist(),
                   iters=r["iters"][:, 0].tolist(), status=int(np.bitwise_or.reduce(r["status"])))
    print(json.dumps(out))


if __name__ == "__main__":
    main()
