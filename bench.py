"""Throughput benchmark of the NEGF transport hot path on GB300.

Workload: the electron ribbon of the headline metric -- single-orbital
nearest-neighbour square lattice, width 32 (n = 32 per slice), 200 device
slices with Anderson disorder U[-0.5, 0.5]|t|, t = -1, 1024 energies on
[-4.2, 4.2]|t|, eta = 1e-6 (synthetic, seeded).  One step = one pass of the
hot path over the whole 1024-point batch: both lead decimations, the
left-to-right RGF sweep and the Caroli trace for every energy, i.e. one
T(E) per (E, q) point ("solve").

    python bench.py [--gpus N] [--steps K] [--warmup W] [--path mixed|fp64]
    python bench.py --impl reference ...   (CPU oracle on the host cores)

Rank 0 prints one JSON line.  `value` = solves/s of the headline path
(default: mixed precision -- FP64-grade lead decimations with their block
products on the tensor cores, FP32 factorisation, double-float refinement:
one sweep for every point and a second for the points whose first
correction was above 3e-5; one CUDA-graph replay a step) with inputs
resident in HBM (CUDA events around each step on the launching stream, L2
flushed before every step); `roofline` = the dominant kernel (the lead
decimations, timed by the library's stage events);
`e2e` = the same through the host-pointer C entry with host buffers, copies
inside the timed region; `compare` = the plain FP64 path on the same batch
(speed-up and the accuracy of the headline T(E) against it).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(workload="tb_ribbon_W32_L200_1024E", n=32, L=200, ne=1024, W=32, t=-1.0,
                disorder=0.5, emin=-4.2, emax=4.2, eta=1e-6, convergence=1e-14)
METRIC = "RGF (omega,q) solves/s (T(E) per point), tb ribbon n=32 L=200, 1024 E"


def flops_per_solve(n, L, I):
    """Algorithmic real flops of one solve: n^3 (40 L + 16) + 2 n^3 (56 I + 24)."""
    return n ** 3 * (40 * L + 16) + 2 * n ** 3 * (56 * I + 24)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return dict(sm_mhz=None, sm_max_mhz=None, reasons=["nvidia-smi unavailable"], samples=0)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return dict(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=smax,
                    reasons=sorted(reasons), samples=len(sm))


def measure_peak(torch, dtype, n):
    """Live cuBLAS GEMM rate (TFLOP/s) used as the roofline denominator."""
    a = torch.randn(n, n, dtype=dtype, device="cuda")
    b = torch.randn(n, n, dtype=dtype, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        torch.cuda.synchronize()
        best = min(best, s.elapsed_time(e) * 1e-3)
    mult = 8 if dtype.is_complex else 2
    return mult * n ** 3 / best / 1e12


def cpu_oracle_rate(E, blocks, p, budget_s=12.0, min_pts=16):
    """Oracle solves/s on the host cores for a bounded sample of the workload:
    the C restatement of the FP64 oracle (oracle/negf_c.c, every host
    thread, one energy per OpenMP iteration); the numpy oracle if the C
    one cannot be built."""
    try:
        from oracle.negf_c import transport_c
        threads = os.cpu_count() or 1

        def solve(Es):
            return transport_c(Es, blocks, p["eta"], p["eta0"], p["convergence"], p["dev_factor"],
                               threads=threads)[2]
        what = "C restatement of the FP64 oracle (oracle/negf_c.c), OpenMP over energies"
        cores = solve(E[:1])
    except (OSError, ImportError, subprocess.CalledProcessError):
        from oracle import negf as N
        try:
            from threadpoolctl import threadpool_info
            cores = max([i.get("num_threads", 1) for i in threadpool_info()] or [1])
        except Exception:  # noqa: BLE001
            cores = os.cpu_count() or 1

        def solve(Es):
            N.transport(Es, blocks, p["eta"], p["eta0"], p["convergence"], p["dev_factor"], want_plus_minus=False)
        what = "numpy restatement of the FP64 oracle (oracle/negf.py)"
    npts = min_pts
    idx = np.linspace(0, len(E) - 1, npts).astype(int)
    t0 = time.perf_counter()
    solve(E[idx])
    dt = time.perf_counter() - t0
    # grow the sample to roughly `budget_s` of CPU work
    if dt < budget_s / 2:
        npts2 = int(min(len(E), max(npts, npts * budget_s / max(dt, 1e-3))))
        idx = np.linspace(0, len(E) - 1, npts2).astype(int)
        t0 = time.perf_counter()
        solve(E[idx])
        dt = time.perf_counter() - t0
        npts = npts2
    return npts / dt, cores, f"{npts} of {len(E)} energies (uniform stride), T_L only, {what}", what


def build_workload():
    from phinfortran_gb300 import systems
    w = WORKLOAD
    b, E, p = systems.tb_ribbon(W=w["W"], L=w["L"], t=w["t"], disorder=w["disorder"], ne=w["ne"],
                                emin=w["emin"], emax=w["emax"], eta=w["eta"], convergence=w["convergence"])
    return b, E, p


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    b, E, p = build_workload()
    vals = []
    info = None
    for i in range(args.warmup + args.steps):
        v, cores, sample, what = cpu_oracle_rate(E, b, p, budget_s=args.ref_budget)
        info = (cores, sample, what)
        if i >= args.warmup:
            vals.append(v)
    v = statistics.median(vals)
    line = dict(metric=METRIC, value=v, unit="solves/s", n_gpus=args.gpus, steps=args.steps,
                warmup=args.warmup, ms_per_step=1e3 * WORKLOAD["ne"] / v, higher_is_better=True,
                scaling="weak", vs_baseline=None, dtype="complex128", data="synthetic (seeded)",
                config=dict(workload=WORKLOAD["workload"], n=32, L=200, energies=1024, eta=1e-6),
                impl="reference",
                cpu_baseline=dict(value=v, unit="solves/s", cores=info[0], kind="port", sample=info[1]),
                e2e=dict(value=v, unit="solves/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0),
                note="reference Fortran/MPI/MKL build is not compilable here (no Fortran, MPI or LAPACK); "
                     f"the timed CPU implementation is the {info[2]} of the path")
    print(json.dumps(line), flush=True)


def time_steps(torch, fn, steps, flush, stream):
    times = []
    for _ in range(steps):
        flush.zero_()                       # evict L2 (256 MB > 129 MB) outside the timed window
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record(stream)
        fn()
        e.record(stream)
        torch.cuda.synchronize()
        times.append(s.elapsed_time(e) * 1e-3)
    return times


def large_block_sample(torch, sizes=((2, 2, 128), (3, 2, 128), (4, 1, 32)), extras=True):
    """Large-block engine on diamond-slab stacks (first + second neighbour
    springs, 28 / 72.6 mass blocks of 10 layers, L = 60): the plain FP64
    path (SIMT FP64 block products), the tensor-core path (the same FP64
    algorithm with every block product on tcgen05 as exact BF16 slice
    products) and the double-float engine.  Each sample keeps the shape of
    the 64 q x 512 omega workload -- many frequencies per transverse k, so
    that the per-q batches of the engine fill the GPU -- at a size that runs
    in seconds: n = 96 (2 transverse k x 128 omega), n = 216 (2 x 128) and
    n = 384 (1 x 32)."""
    from phinfortran_gb300 import systems as S, transport_tdb
    out = []
    for nc, nk, ne in sizes:
        kp = list(range(0, 64, 64 // nk))[:nk]
        b, E, p, aux = S.diamond_phonon(nc=nc, L=60, kpoints=kp)
        Es = E[np.linspace(10, 500, ne).astype(int)]
        Eall = np.tile(Es, nk)
        q = np.repeat(np.arange(nk, dtype=np.int32), ne)
        res = {}
        for prec in ("fp64", "tc", "df64"):
            transport_tdb(Eall[:1], b, qidx=q[:1], want_transr=False, precision=prec, **p)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = transport_tdb(Eall, b, qidx=q, want_transr=False, check=False, precision=prec, **p)
            torch.cuda.synchronize()
            res[prec] = (time.perf_counter() - t0, r)
        n = aux["n"]
        I = float(res["fp64"][1]["iters"][:, 0].mean())
        fl = flops_per_solve(n, 60, I) * Eall.size
        T64 = res["fp64"][1]["transl"]
        dev = {k: float((np.abs(res[k][1]["transl"] - T64) / np.maximum(np.abs(T64), 1e-3)).max())
               for k in ("tc", "df64")}
        out.append(dict(n=n, L=60, points=int(Eall.size), mean_decimation_iters=I,
                        fp64_solves_per_s=Eall.size / res["fp64"][0],
                        tc_solves_per_s=Eall.size / res["tc"][0],
                        df64_solves_per_s=Eall.size / res["df64"][0],
                        tc_speedup_vs_fp64=res["fp64"][0] / res["tc"][0],
                        df64_speedup_vs_fp64=res["fp64"][0] / res["df64"][0],
                        fp64_tflops_algorithmic=fl / res["fp64"][0] / 1e12,
                        tc_tflops_algorithmic=fl / res["tc"][0] / 1e12,
                        tc_max_rel_dev_from_fp64=dev["tc"], df64_max_rel_dev_from_fp64=dev["df64"],
                        status_nonzero={k: int((res[k][1]["status"] != 0).sum()) for k in res},
                        note="host-pointer call (blocks copied to the device inside the timed region); "
                             "deviation = max |T - T64| / max(|T64|, 1e-3); built-in panel width and batch"))
        if n == 216 and extras:
            # the autotuner on a 48-point subsample of this problem (tensor-core
            # arithmetic): panel width of the blocked inverse x batch
            import tempfile
            from phinfortran_gb300.autotune import autotune_tiled, set_tuning
            sel = np.linspace(0, Eall.size - 1, 48).astype(int)
            with tempfile.TemporaryDirectory() as td:
                best = autotune_tiled(Eall[sel], b, precision="tc", panels=(8, 16, 32), batches=(16, 48),
                                      cache=os.path.join(td, "tune.json"), qidx=q[sel], **p)
            set_tuning(0, 0)
            out[-1]["autotune"] = dict(sample_points=48, panel=best["panel"], batch=best["batch"],
                                       tuned_s=best["seconds"], default_s=best["default_seconds"],
                                       candidates=[(c["panel"], c["batch"], c["seconds"]) for c in best["candidates"]],
                                       note="panel 0 / batch 0 = the built-in choice")
    if extras:
        out.append(circular_sample(torch))
    return out


def circular_sample(torch, nc=3, ne=64):
    """Block-circulant leads (circular_flag = 1): the diamond slab at the
    transverse Gamma point has nc x nc block-circulant lead matrices; the
    lead surface Green's functions through circular_g (K = nc^2 small
    decimations of 24 x 24 per point) against the decimation of the full
    n x n lead matrices, tensor-core block products, L = 60, ne points."""
    from phinfortran_gb300 import systems as S, transport_tdb
    b, E, p, aux = S.diamond_phonon(nc=nc, L=60, nk_side=1, ne=ne)
    bq = {k: v[0] for k, v in b.items()}
    res = {}
    for mode in ("full", "circular"):
        kw = dict(circular=(nc, nc, [2.0 * np.pi] * 4)) if mode == "circular" else {}
        transport_tdb(E[:2], bq, want_transr=False, precision="tc", **kw, **p)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = transport_tdb(E, bq, want_transr=False, check=False, precision="tc", **kw, **p)
        torch.cuda.synchronize()
        res[mode] = (time.perf_counter() - t0, r)
    Tf, Tc = res["full"][1]["transl"], res["circular"][1]["transl"]
    return dict(n=aux["n"], L=60, points=int(E.size), circular=dict(n_bloch_y=nc, n_bloch_x=nc, small_block=24),
                full_solves_per_s=E.size / res["full"][0], circular_solves_per_s=E.size / res["circular"][0],
                circular_speedup=res["full"][0] / res["circular"][0],
                max_rel_dev=float((np.abs(Tc - Tf) / np.maximum(np.abs(Tf), 1e-3)).max()),
                status_nonzero={k: int((res[k][1]["status"] != 0).sum()) for k in res},
                note="host-pointer call, tensor-core products; deviation = max |T_circ - T_full| / max(|T_full|, 1e-3)")


def tc_zgemm_rate(torch, m=384, batch=64, reps=5):
    """The batched tensor-core ZGEMM of the large-block engine
    (pf_tc_zgemm_dev, FP64-grade: 9 BF16 slices an operand, the 45 slice
    pairs with s + t <= 10, each a real GEMM of 8 m n k flops on the
    interleaved embedding) on m = n = k, batch products, inputs of 3 x 151 MB
    (above L2).  CUDA events around each call on its stream (slicing,
    exponent scans, products and assembly), after 3 warm-up calls."""
    import ctypes as C
    from phinfortran_gb300 import _abi
    lib = _abi.load()
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn(batch * m * m * 2, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(batch * m * m * 2, dtype=torch.float64, device="cuda", generator=g)
    Cm = torch.zeros(batch * m * m * 2, dtype=torch.float64, device="cuda")
    ws = lib.pf_tc_zgemm_workspace_size(m, m, m, batch, 0, 0)
    work = torch.empty(ws, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream()
    s2 = m * m

    def call():
        rc = lib.pf_tc_zgemm_dev(ord("N"), ord("N"), m, m, m, 1.0, A.data_ptr(), m, s2, B.data_ptr(), m, s2, 0.0,
                                 Cm.data_ptr(), m, s2, batch, work.data_ptr(), ws, C.c_void_p(st.cuda_stream))
        if rc != 0:
            raise _abi.PFError(rc, lib.pf_tc_last_error().decode(errors="replace"))
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        call()
        e1.record(st)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    t = statistics.median(times)
    fl = 8.0 * m * m * m * batch
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    bf16_peak = float(peaks.get("bf16_tflops", 1900.0))
    bf16 = 45 * fl / t / 1e12
    return dict(m=m, n=m, k=m, batch=batch, ms_per_call=t * 1e3, fp64_equivalent_tflops=fl / t / 1e12,
                bf16_tensor_tflops=bf16, bf16_peak_tflops=bf16_peak, frac_of_bf16_peak=bf16 / bf16_peak,
                slice_pairs=45, note="whole call (slicing + products + FP64 assembly); bf16 = 45 pair products x "
                                     "8 m n k flops a product; peak: dense bf16 burst of MEASURED_PEAKS.json")


def gradient_ratio(torch, flush, stream, steps):
    """Adjoint gradient (d kappa / d every block) vs one forward sweep on the
    simple-cubic 4x4x40 bar (n=48, L=40), masses U[1,3], springs U[0.8,1.2],
    1024 frequencies, Landauer weights at T=300 (arb. units)."""
    from phinfortran_gb300 import DeviceTransport, systems as S
    from phinfortran_gb300.gradients import DeviceGradient, landauer_weights
    b, E, p, aux = S.sc_phonon(nx=4, ny=4, L=40, ne=1024, mass_range=(1.0, 3.0), bond_range=(0.8, 1.2),
                               seed_index=4)
    Ed = torch.from_numpy(E).cuda()
    w = torch.from_numpy(landauer_weights(aux["omega"], 300.0)).cuda()
    f64 = DeviceTransport(b, E.size, precision="fp64", **p)
    mix = DeviceTransport(b, E.size, precision="mixed", **p)
    gr = DeviceGradient(b, E.size, ckpt=0, arith="df64", **p)
    gr_all = DeviceGradient(b, E.size, ckpt=1, arith="df64", **p)
    gr64 = DeviceGradient(b, E.size, ckpt=0, arith="fp64", **p)
    out = {}
    for name, fn in (("fwd_fp64", lambda: f64.run(Ed, stream=stream)), ("fwd_mixed", lambda: mix.run(Ed, stream=stream)),
                     ("grad", lambda: gr.run(Ed, w, stream=stream)),
                     ("grad_store_all", lambda: gr_all.run(Ed, w, stream=stream)),
                     ("grad_fp64", lambda: gr64.run(Ed, w, stream=stream))):
        fn()
        torch.cuda.synchronize()
        t = time_steps(torch, fn, steps, flush, stream)
        out[name + "_ms"] = 1e3 * sum(t) / len(t)
    Tg = gr.transl[:E.size].cpu().numpy()
    T64 = f64.transl[:E.size].cpu().numpy()
    torch.cuda.synchronize()
    M = {k: v[0] for k, v in gr.sensitivities().items()}
    M64 = {k: v[0] for k, v in gr64.sensitivities().items()}
    dev = max(float(np.abs(M[k] - M64[k]).max() / max(np.abs(M64[k]).max(), 1e-300)) for k in M if M[k].size)
    return dict(workload="simple-cubic phonon bar 4x4x40 (n=48, L=40), masses U[1,3], springs U[0.8,1.2], "
                         "1024 omega, kappa at T=300",
                grad_over_fwd_fp64=out["grad_ms"] / out["fwd_fp64_ms"],
                grad_over_fwd_mixed=out["grad_ms"] / out["fwd_mixed_ms"],
                grad_store_all_over_fwd_mixed=out["grad_store_all_ms"] / out["fwd_mixed_ms"],
                grad_fp64_over_fwd_fp64=out["grad_fp64_ms"] / out["fwd_fp64_ms"],
                grad_T_max_abs_dev_from_fp64=float(np.abs(Tg - T64).max()),
                grad_sensitivity_max_rel_dev_df64_vs_fp64=dev,
                note="grad = adjoint kernel in double-float arithmetic (forward T plus the weighted sensitivities "
                     "of every device block) with the left-connected factors checkpointed every ceil(sqrt(L+2)) = 7 "
                     "layers and recomputed; grad_store_all keeps every layer; grad_fp64 = the same checkpointed "
                     "kernel in FP64", **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--path", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--refine", type=int, default=2,
                    help="maximum refinement sweeps of the mixed path (sweeps after the first are adaptive)")
    ap.add_argument("--ref-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the FP64 comparison path (accuracy and speed-up fields)")
    ap.add_argument("--no-grad", action="store_true", help="skip the gradient / forward cost ratio")
    ap.add_argument("--no-large", action="store_true", help="skip the large-block (diamond slab) sample")
    ap.add_argument("--no-graph", action="store_true", help="time direct launches instead of a CUDA-graph replay")
    ap.add_argument("--energies", type=int, default=0,
                    help="use only N energies of the workload (profiling runs)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from phinfortran_gb300 import DeviceTransport, transport_tdb
    from phinfortran_gb300.transport import TdbBlocks, fortran_block

    b, E, p = build_workload()
    if args.energies:
        E = E[np.linspace(0, len(E) - 1, args.energies).astype(int)]
    npts = len(E)
    Ed = torch.from_numpy(E).to("cuda")
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(t):
        if ws > 1:
            tt = torch.tensor([t], device="cuda", dtype=torch.float64)
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            return tt.item()
        return t

    main_dt = DeviceTransport(b, npts, want_transr=False, precision=args.path, refine_iters=args.refine, **p)
    for _ in range(args.warmup):
        main_dt.run(Ed, stream=stream)
    torch.cuda.synchronize()
    iters = main_dt.iters[:npts].float().mean().item()
    status = main_dt.status[:npts].cpu().numpy()
    T_main = main_dt.transl[:npts].cpu().numpy().copy()

    # the step is captured once into a CUDA graph and replayed (no host work
    # inside the timed region); the direct launch sequence is timed beside it
    graph = None
    if not args.no_graph:
        try:
            graph = main_dt.capture(Ed)
            graph.replay()
            torch.cuda.synchronize()
            if not np.array_equal(main_dt.transl[:npts].cpu().numpy(), T_main):
                graph = None
        except RuntimeError:
            graph = None
    step_fn = (lambda: graph.replay()) if graph is not None else (lambda: main_dt.run(Ed, stream=stream))

    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    times = time_steps(torch, step_fn, args.steps, flush, stream)
    barrier()
    clk = clocks.stop()
    t_step = max_over_ranks(sum(times) / len(times))
    value = ws * npts / t_step
    t_direct = None
    if graph is not None:
        td = time_steps(torch, lambda: main_dt.run(Ed, stream=stream), max(1, min(args.steps, 3)), flush, stream)
        t_direct = sum(td) / len(td)
    # stage times of the mixed pipeline (CUDA events recorded by the library on
    # the launch stream around the lead-decimation kernel): the roofline of
    # the dominant kernel is taken from these
    stage_ms = None
    if args.path == "mixed":
        import ctypes as C
        from phinfortran_gb300 import _abi
        lib = _abi.load()
        lib.pf_mixed_stage_timing(1)
        acc = np.zeros(3)
        nrun = max(1, min(args.steps, 3))
        buf = (C.c_float * 3)()
        for _ in range(nrun):
            flush.zero_()
            main_dt.run(Ed, stream=stream)
            if lib.pf_mixed_stage_times(buf, 3) != 3:
                acc = None
                break
            acc += np.array(buf[:3], dtype=float)
        lib.pf_mixed_stage_timing(0)
        if acc is not None:
            stage_ms = dict(zip(("setup", "leads", "sweeps"), (acc / nrun).tolist()))

    # ---- FP64 comparison path: speed-up and accuracy of the headline path ----
    compare = None
    if not args.no_compare:
        f64 = DeviceTransport(b, npts, want_transr=False, precision="fp64", **p) if args.path != "fp64" else main_dt
        for _ in range(1 if f64 is not main_dt else 0):
            f64.run(Ed, stream=stream)
        torch.cuda.synchronize()
        t64 = time_steps(torch, lambda: f64.run(Ed, stream=stream), max(1, min(args.steps, 3)), flush, stream)
        T64 = f64.transl[:npts].cpu().numpy().copy()
        # FP64 conditioning of every point: rerun with every block perturbed by ~1e-15 relative
        rng = np.random.default_rng(123)
        bp = {k: np.asarray(v) * (1 + 1e-15 * rng.standard_normal(np.shape(v))) for k, v in b.items()}
        fp = DeviceTransport(bp, npts, want_transr=False, precision="fp64", **p)
        fp.run(Ed, stream=stream)
        torch.cuda.synchronize()
        floor = np.abs(fp.transl[:npts].cpu().numpy() - T64)
        rel = np.abs(T_main - T64) / np.maximum(np.abs(T64), 1e-3)
        good = floor / np.maximum(np.abs(T64), 1e-3) <= 1e-10
        compare = dict(
            fp64_solves_per_s=ws * npts / max_over_ranks(sum(t64) / len(t64)),
            fp64_ms_per_step=1e3 * sum(t64) / len(t64),
            speedup_vs_fp64=(ws * npts / t_step) / (ws * npts / max_over_ranks(sum(t64) / len(t64))),
            accuracy=dict(reference="FP64 GPU path, same energies", metric="|T-T64|/max(|T64|,1e-3)",
                          median=float(np.median(rel)), q99=float(np.quantile(rel, 0.99)), max=float(rel.max()),
                          frac_le_1e_8=float((rel <= 1e-8).mean()),
                          fp64_conditioned_points=int(good.sum()),
                          frac_le_1e_8_where_fp64_reproducible=float((rel[good] <= 1e-8).mean()) if good.any() else None,
                          max_where_fp64_reproducible=float(rel[good].max()) if good.any() else None,
                          note="points are 'fp64 reproducible' when a 1e-15 relative perturbation of the inputs "
                               "moves the FP64 result by <= 1e-10 relative"))
        # the faster lead arithmetics of the mixed path, for the record
        if args.path == "mixed":
            variants = {}
            for lead in ("split", "df64"):
                dv = DeviceTransport(b, npts, want_transr=False, precision="mixed", refine_iters=args.refine,
                                     lead_arith=lead, **p)
                dv.run(Ed, stream=stream)
                torch.cuda.synchronize()
                tv = time_steps(torch, lambda: dv.run(Ed, stream=stream), max(1, min(args.steps, 3)), flush, stream)
                rv = np.abs(dv.transl[:npts].cpu().numpy() - T64) / np.maximum(np.abs(T64), 1e-3)
                variants[lead] = dict(ms_per_step=1e3 * sum(tv) / len(tv), solves_per_s=npts / (sum(tv) / len(tv)),
                                      frac_le_1e_8=float((rv <= 1e-8).mean()),
                                      frac_le_1e_8_where_fp64_reproducible=float((rv[good] <= 1e-8).mean()),
                                      max_where_fp64_reproducible=float(rv[good].max()))
                del dv
            compare["lead_arith_variants"] = variants
            compare["lead_arith_note"] = ("headline: FP64-grade lead decimations (block products on tcgen05 as "
                                          "exact BF16 slice products, FP64 inverse); split = first 8 decimation "
                                          "steps in FP64 then double-float; df64 = double-float decimations")

    # ---- gradient cost vs forward cost on the differentiable-conductance workload ----
    grad = None
    if not args.no_grad:
        grad = gradient_ratio(torch, flush, stream, max(1, min(args.steps, 2)))

    # ---- large blocks: diamond slab stacks (n = 96, 216; L = 60) ----
    large = None
    tcz = None
    if not args.no_large:
        large = large_block_sample(torch)
        tcz = tc_zgemm_rate(torch)

    # ---- end to end through the host-pointer C entry ----
    nq, dims, arrs = TdbBlocks.from_dict(b).stacked()
    h2d = sum(fortran_block(v).nbytes for v in arrs.values()) + E.nbytes
    d2h = npts * 8 + npts * 4 + npts * 8      # transl, status, iterations
    call = lambda: transport_tdb(E, b, want_transr=False, precision=args.path, refine_iters=args.refine, **p)
    for _ in range(0 if args.no_e2e else 2):
        call()
    barrier()
    e2e_t = [float("inf")] if args.no_e2e else []
    for _ in range(0 if args.no_e2e else args.steps):
        t0 = time.perf_counter()
        call()
        e2e_t.append(time.perf_counter() - t0)
    barrier()
    t_e2e = max_over_ranks(sum(e2e_t) / len(e2e_t))
    e2e_value = ws * npts / t_e2e

    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return

    n, L = WORKLOAD["n"], WORKLOAD["L"]
    fl = flops_per_solve(n, L, iters) * npts
    achieved = fl / t_step / 1e12
    # denominator: the measured dense bf16 tensor-core peak (MEASURED_PEAKS.json,
    # burst figure); beside it the peak of the pipe this path actually runs on
    mp_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    bf16_peak = None
    if os.path.exists(mp_path):
        with open(mp_path) as f:
            bf16_peak = json.load(f).get("bf16_tflops")
    peak_label = "of measured" if bf16_peak else "of fallback"
    if not bf16_peak:
        bf16_peak = 1900.0
    if args.path == "fp64":
        pipe_peak = measure_peak(torch, torch.complex128, 2048)
        pipe = "fp64"
        pipe_src = "cuBLAS ZGEMM 2048^3 measured live on this GPU (FP64 pipe)"
        kernel = "transport_kernel<double>"
    else:
        torch.backends.cuda.matmul.allow_tf32 = False
        pipe_peak = measure_peak(torch, torch.complex64, 4096)
        pipe = "fp32-simt"
        pipe_src = ("cuBLAS CGEMM 4096^3 (FP32 SIMT, TF32 off) measured live on this GPU: the sweeps of the "
                    "32-wide mixed pipeline run on the FP32 pipe (FP32 and double-float arithmetic); the lead "
                    "decimations on the tensor cores and the FP64 pipe (see roofline.kernel)")
        kernel = ("mixed pipeline per step (one CUDA-graph replay): leads_tc_kernel (FP64-grade decimation, "
                  "its block products on tcgen05, one CTA per SM) + layer_kernel (warp per point: FP32 LU, back "
                  "substitution, refinement corrections, Caroli; the adaptive second sweep with a CTA per listed "
                  "point) + residual_kernel; achieved = F per step / step time")
    step_roof = dict(achieved=achieved, unit="TFLOP/s", frac_of_bf16=achieved / bf16_peak, pipe=pipe,
                     pipe_peak=pipe_peak, pipe_frac=achieved / pipe_peak, pipe_peak_source=pipe_src, kernel=kernel,
                     algorithmic_flops_per_launch=fl, flops_formula="n^3 (40 L + 16) + 2 n^3 (56 I + 24)",
                     mean_decimation_iters=iters, traffic=None)
    prof = os.path.join(ROOT, "profiles", f"{args.path}_kernel_tb_ribbon.json")
    if os.path.exists(prof):
        with open(prof) as f:
            pj = json.load(f)
        if args.path == "fp64" or pj.get("refine_iters") == args.refine:
            step_roof["traffic"] = pj.get("dram_bytes_per_launch_scaled")
            step_roof["traffic_source"] = pj.get("source")
    if args.path == "mixed" and stage_ms is not None:
        # dominant kernel: the lead decimations (one launch a step)
        fl_leads = 2.0 * n ** 3 * (56 * iters + 24) * npts
        zgemm_peak = measure_peak(torch, torch.complex128, 2048)
        t_leads = stage_ms["leads"] * 1e-3
        ach = fl_leads / t_leads / 1e12
        roof = dict(bound="tensor", achieved=ach, peak=bf16_peak, unit="TFLOP/s", frac=ach / bf16_peak, traffic=None,
                    peak_source=f"dense bf16 burst {peak_label} (MEASURED_PEAKS.json bf16_tflops)",
                    kernel="leads_tc_kernel: FP64-grade Lopez-Sancho decimations, block products on tcgen05 as "
                           "exact BF16 slice products (36 pair products a call, two calls a step), FP64 look-ahead "
                           "inverse; achieved = FP64-equivalent decimation flops / kernel time",
                    launch_ms=stage_ms["leads"], timing="CUDA events on the launch stream around the kernel, "
                    "recorded by the library (pf_mixed_stage_times), mean of direct calls after the timed region",
                    algorithmic_flops_per_launch=fl_leads, flops_formula="2 n^3 (56 I + 24) per point (the decimation "
                    "term of F)", fp64_equivalent_frac_of_zgemm=ach / zgemm_peak, zgemm_peak=zgemm_peak, stage_ms=stage_ms, step=step_roof)
        lj = os.path.join(ROOT, "profiles", "leads_tc_kernel_tb_ribbon.json")
        if os.path.exists(lj):
            with open(lj) as f:
                pj = json.load(f)
            roof["traffic"] = pj.get("dram_bytes_per_launch_scaled")
            roof["traffic_source"] = pj.get("source")
    else:
        roof = dict(bound="tensor", achieved=achieved, peak=bf16_peak, unit="TFLOP/s", frac=achieved / bf16_peak,
                    traffic=step_roof.get("traffic"), traffic_source=step_roof.get("traffic_source"),
                    peak_source=f"dense bf16 burst {peak_label} (MEASURED_PEAKS.json bf16_tflops)",
                    pipe=pipe, pipe_peak=pipe_peak, pipe_frac=achieved / pipe_peak, pipe_peak_source=pipe_src,
                    kernel=kernel, algorithmic_flops_per_launch=fl,
                    flops_formula="n^3 (40 L + 16) + 2 n^3 (56 I + 24)", mean_decimation_iters=iters)

    cpu = None
    if not args.no_cpu_baseline:
        v, cores, sample, _ = cpu_oracle_rate(E, b, p)
        cpu = dict(value=v, unit="solves/s", cores=cores, kind="port", sample=sample)

    if args.path == "fp64":
        launches_per_step = 2                         # lead-mirror check + transport_kernel
    else:
        # 8 block conversions + 7 ELL builds + lead-mirror check + leads_tc_kernel + layer_kernel (factor)
        # + the first refinement sweep (residual_kernel + layer_kernel) + each later, adaptive sweep
        # (refine_select_kernel + residual_kernel + layer_kernel) + point-energy kernel + layer_kernel (Caroli)
        sweeps = (2 + 3 * (args.refine - 1) + 1) if args.refine else 0
        launches_per_step = 8 + 7 + 1 + 1 + 1 + sweeps + 1
    line = dict(metric=METRIC, value=value, unit="solves/s", n_gpus=ws, steps=args.steps, warmup=args.warmup,
                ms_per_step=t_step * 1e3, higher_is_better=True, scaling="weak", vs_baseline=None,
                dtype="complex128 (fp64)" if args.path == "fp64" else
                ("complex: FP64-grade leads (tcgen05 bf16 slice products, fp64 inverse) + fp32 factorisation "
                 "+ double-float refinement"),
                data="synthetic (seeded PCG64)",
                config=dict(workload=WORKLOAD["workload"], n=n, L=L, energies=npts, eta=1e-6, path=args.path,
                            refine_iters=args.refine if args.path == "mixed" else None,
                            l2="flushed (256 MB write) before every timed step", parallelism=f"replicas x{ws}",
                            timed="one CUDA-graph replay per step" if graph is not None else "direct launches"),
                direct_launch_ms_per_step=None if t_direct is None else t_direct * 1e3,
                e2e=dict(value=e2e_value, unit="solves/s", h2d_bytes_per_step=int(h2d), d2h_bytes_per_step=int(d2h),
                         entry="pf_transport_tdb_mixed" if args.path == "mixed" else "pf_transport_tdb"),
                roofline=roof, cpu_baseline=cpu, compare=compare, gradient=grad, large_blocks=large, tc_zgemm=tcz,
                clocks=dict(sm_mhz=clk["sm_mhz"], sm_max_mhz=clk["sm_max_mhz"], reasons=clk["reasons"]),
                gpu_launches=launches_per_step * args.steps, status_nonzero=int((status != 0).sum()))
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
