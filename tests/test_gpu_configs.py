"""Parity at the shapes of the benchmark configurations that the smaller
GPU tests do not reach: all 256 frequencies of the simple-cubic bar
(n = 48, L = 20), the adjoint at the full differentiable-conductance size
(n = 48, L = 40), the 4 x 4-cell diamond slab (n = 384) and the 3-orbital
ribbon of width 256 (n = 768).  The large blocks are checked in all three
arithmetics of the large-block engine (FP64 products, tensor-core slice
products, double-float); the n = 768 case against the FP64 GPU path, whose
engine the oracle pins at the smaller sizes (the CPU oracle would take
minutes per energy there)."""
import numpy as np
import pytest

from oracle import adjoint as A
from oracle import negf as N
from phinfortran_gb300 import systems as S
from phinfortran_gb300 import transport_tdb
from phinfortran_gb300.gradients import transport_grad

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1.0)


def test_sc_bar_all_256_frequencies(cuda_ready):
    """cfg1 shape: 4 x 4 cross-section (n = 48), L = 20, masses U[1, 2],
    all 256 frequencies, FP64 path vs the oracle (T_L and T_R)."""
    b, E, p, _ = S.sc_phonon(ne=256)
    r = transport_tdb(E, b, want_transr=True, **p)
    o = N.transport(E, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"])
    assert (r["status"] == 0).all()
    assert np.median(rel(r["transl"], o["transl"])) < 1e-11
    assert rel(r["transl"], o["transl"]).max() < 1e-8
    assert rel(r["transr"], o["transr"]).max() < 1e-8
    assert np.abs(r["iters"][:, 0] - o["iters_left"]).max() <= 1


@pytest.mark.parametrize("shape", ["cfg1", "cfg4"])
def test_mixed_sc_bar_n48(cuda_ready, shape):
    """The mixed path on the 48-wide phonon bars (the fused kernel; the
    default lead arithmetic is double-float there): every frequency where
    FP64 is reproducible to 1e-10 within 1e-8 of the FP64 GPU path (cfg1:
    all 256 frequencies of the 4 x 4 x 20 bar; cfg4: 256 of the 1024 of the
    4 x 4 x 40 bar)."""
    import torch
    from phinfortran_gb300 import DeviceTransport
    if shape == "cfg1":
        b, E, p, _ = S.sc_phonon(ne=256)
    else:
        b, E, p, _ = S.sc_phonon(nx=4, ny=4, L=40, ne=1024, mass_range=(1.0, 3.0), bond_range=(0.8, 1.2),
                                 seed_index=4)
        E = E[::4]
    Ed = torch.from_numpy(E).cuda()
    T = {}
    rng = np.random.default_rng(3)
    bp = {k: np.asarray(v) * (1 + 1e-15 * rng.standard_normal(np.shape(v))) for k, v in b.items()}
    for key, blocks, prec in (("fp64", b, "fp64"), ("pert", bp, "fp64"), ("mixed", b, "mixed")):
        dt = DeviceTransport(blocks, E.size, precision=prec, **p)
        dt.run(Ed)
        torch.cuda.synchronize()
        assert (dt.status[:E.size].cpu().numpy() == 0).all()
        T[key] = dt.transl[:E.size].cpu().numpy().copy()
    r = lambda a: np.abs(a - T["fp64"]) / np.maximum(np.abs(T["fp64"]), 1e-3)
    good = r(T["pert"]) <= 1e-10
    assert good.mean() > 0.9
    assert r(T["mixed"])[good].max() <= 1e-8


@pytest.mark.parametrize("arith", ["fp64", "df64"])
def test_adjoint_at_full_conductance_size(cuda_ready, arith):
    """cfg4 shape: 4 x 4 x 40 bar (n = 48, L = 40), masses U[1, 3], springs
    U[0.8, 1.2]; 16 frequencies; checkpointed adjoint (ceil(sqrt(42)) = 7)
    vs the oracle adjoint."""
    b, E, p, aux = S.sc_phonon(nx=4, ny=4, L=40, ne=1024, mass_range=(1.0, 3.0), bond_range=(0.8, 1.2),
                               seed_index=4)
    Es = E[np.linspace(20, 1000, 16).astype(int)]
    w = np.linspace(0.5, 1.5, Es.size)
    T, M, st = transport_grad(Es, b, w, ckpt=0, arith=arith, **p)
    To, Mo = A.transport_and_sensitivities(Es, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"])
    assert (st == 0).all()
    tol_t, tol_m = (1e-9, 1e-8) if arith == "fp64" else (1e-8, 1e-6)
    assert rel(T, To).max() < tol_t
    for k in ("Hd", "Hdv", "Hld", "Hrd"):
        ref = np.tensordot(w, Mo[k], axes=(0, 0))
        got = M[k][0]
        assert np.abs(got - ref).max() <= tol_m * np.abs(ref).max(), k


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("tc", 1e-9), ("df64", 1e-7)])
def test_diamond_n384_against_oracle(cuda_ready, precision, tol):
    """cfg3's largest cross-section: 4 x 4 conventional cells (n = 384), a
    28 / 72.6 mass interface, L = 4, one transverse q, two frequencies."""
    b, E, p, aux = S.diamond_phonon(nc=4, L=4, nk_side=8, ne=12, kpoints=[9], block=2)
    bq = {k: v[0] for k, v in b.items()}
    Es = E[[4, 8]]
    r = transport_tdb(Es, bq, want_transr=False, precision=precision, **p)
    o = N.transport(Es, bq, p["eta"], p["eta0"], p["convergence"], p["dev_factor"])
    assert (r["status"] == 0).all()
    assert rel(r["transl"], o["transl"]).max() < tol, rel(r["transl"], o["transl"])
    assert np.abs(r["iters"][:, 0] - o["iters_left"]).max() <= 1


def test_ribbon3_n768_tensor_core_vs_fp64(cuda_ready):
    """cfg5's cross-section: 3-orbital ribbon of width 256 (n = 768), L = 6,
    two energies: the tensor-core products give the FP64 path's T within
    1e-9 or 20x FP64's own noise floor there (the change of the FP64 T when
    every input block is perturbed by 1e-15 relative), relative to
    max(|T|, 1)."""
    b, E, p = S.tb_ribbon3(W=256, L=6, ne=4096, energies=[1100, 2900])
    r64 = transport_tdb(E, b, want_transr=False, precision="fp64", **p)
    rtc = transport_tdb(E, b, want_transr=False, precision="tc", **p)
    rng = np.random.default_rng(7)
    bp = {k: np.asarray(v) * (1 + 1e-15 * rng.standard_normal(np.shape(v))) for k, v in b.items()}
    r64p = transport_tdb(E, bp, want_transr=False, precision="fp64", **p)
    assert (r64["status"] == 0).all() and (rtc["status"] == 0).all()
    floor = rel(r64p["transl"], r64["transl"])
    err = rel(rtc["transl"], r64["transl"])
    assert np.all(err <= np.maximum(1e-9, 20 * floor)), (err, floor)
    assert np.abs(rtc["iters"][:, 0] - r64["iters"][:, 0]).max() <= 1
