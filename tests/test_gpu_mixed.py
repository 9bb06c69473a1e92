"""GPU accuracy of the mixed-precision path (double-float leads, FP32
factorisation, double-float refinement) against the FP64 oracle, through
the C ABI (pf_transport_tdb_mixed)."""
import numpy as np
import pytest

from oracle import negf as N
from phinfortran_gb300 import systems as S
from phinfortran_gb300 import transport_tdb
from tests.sisi_case import fp64_noise_floor, golden_close, sisi_blocks, sisi_params

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-3)


def test_mixed_sc_phonon_meets_1e8(cuda_ready):
    b, E, p, _ = S.sc_phonon(ne=256)
    Es = E[::8]
    o = N.transport(Es, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"])
    r0 = transport_tdb(Es, b, precision="mixed", refine_iters=0, **p)
    r1 = transport_tdb(Es, b, precision="mixed", refine_iters=1, **p)
    e0, e1 = rel(r0["transl"], o["transl"]), rel(r1["transl"], o["transl"])
    assert (r1["status"] == 0).all()
    # FP32 alone is ~1e-7; one double-float refinement sweep reaches < 1e-8 everywhere
    assert np.median(e1) < np.median(e0) / 100
    assert e1.max() <= 1e-8, e1.max()
    # decimation iteration counts match the FP64 stopping rule
    assert np.abs(r1["iters"][:, 0] - o["iters_left"]).max() <= 1


def test_mixed_tb_ribbon_against_oracle(cuda_ready):
    """Benchmark workload (n=32, L=200): error relative to the FP64 conditioning."""
    b, E, p = S.tb_ribbon()
    Es = E[::16]
    r1 = transport_tdb(Es, b, precision="mixed", refine_iters=1, **p)
    r2 = transport_tdb(Es, b, precision="mixed", refine_iters=2, **p)
    o, pert = fp64_noise_floor(Es, b, p)
    # FP64 noise floor of a point: input-perturbation sensitivity or the
    # disagreement of the oracle's two sweeps, whichever is larger
    floor = np.maximum(pert, np.abs(o["transl"] - o["transr"]))
    # double-float carries ~2^-48 per operation (32x FP64's unit roundoff)
    tol = np.maximum(1e-8 * np.maximum(np.abs(o["transl"]), 1e-3), 100 * floor)
    ok = {}
    for k, r in (("r1", r1), ("r2", r2)):
        assert (r["status"] == 0).all()
        d = np.abs(r["transl"] - o["transl"])
        e = rel(r["transl"], o["transl"])
        assert np.median(e) < 1e-8
        assert (e <= 1e-8).mean() >= 0.75
        assert (d <= tol).mean() >= 0.95, np.sort(d / tol)[-5:]
        ok[k] = (d <= tol).mean()
    assert ok["r2"] >= ok["r1"]
    # the second sweep is adaptive: it changes some points and leaves the
    # points whose first correction was small bit-identical
    same = r2["transl"] == r1["transl"]
    assert 0 < same.sum() < same.size, same.sum()


def test_mixed_sisi_against_reference_output(cuda_ready, sisi):
    ik = 24
    b = sisi_blocks(sisi, ik)
    E = sisi["E"]
    zf = np.zeros(E.size, np.int32)
    zf[0] = 1
    r = transport_tdb(E, b, precision="mixed", refine_iters=2, zero_flag=zf, **sisi_params(sisi))
    ok, ad, q99 = golden_close(r["transl"], sisi["transl_tot"][:, ik], abs_tol=1e-6, rel_q99=1e-7)
    assert ok, (ad, q99)
    assert r["transl"][0] == 0.0


def test_mixed_edge_shapes(cuda_ready):
    """Uneven lead/device widths and a single device layer."""
    rng = np.random.default_rng(7)
    n, nl, nr = 6, 4, 5

    def herm(m):
        a = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
        return a + a.conj().T

    for L in (1, 3):
        Hd = np.array([herm(n) for _ in range(L)])
        Hdv = rng.normal(size=(L - 1, n, n)) * 0.5
        blocks = dict(HL=herm(nl), HLv=rng.normal(size=(nl, nl)) * 0.5, HR=herm(nr),
                      HRv=rng.normal(size=(nr, nr)) * 0.5, Hd=Hd, Hdv=Hdv,
                      Hld=rng.normal(size=(nl, n)) * 0.5, Hrd=rng.normal(size=(nr, n)) * 0.5)
        E = np.linspace(-3, 3, 13)
        r = transport_tdb(E, blocks, eta=0.0, eta0=1e-3, convergence=1e-12, dev_factor=1.0,
                          precision="mixed", refine_iters=2)
        o = N.transport(E, blocks, 0.0, 1e-3, 1e-12, 1.0)
        assert np.abs(r["transl"] - o["transl"]).max() < 1e-9, L


def test_mixed_tensor_core_leads_of_two_widths(cuda_ready):
    """The tensor-core lead decimations with a 28-wide left lead and a
    32-wide right lead in the same call (the operand tiles are re-zeroed
    when the block size changes from one product to the next), random
    Hermitian blocks, against the oracle."""
    rng = np.random.default_rng(11)
    n, nl, nr, L = 30, 28, 32, 4

    def herm(m):
        a = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
        return (a + a.conj().T) * 0.5

    blocks = dict(HL=herm(nl), HLv=rng.normal(size=(nl, nl)) * 0.3, HR=herm(nr),
                  HRv=rng.normal(size=(nr, nr)) * 0.3, Hd=np.array([herm(n) for _ in range(L)]),
                  Hdv=rng.normal(size=(L - 1, n, n)) * 0.3, Hld=rng.normal(size=(nl, n)) * 0.3,
                  Hrd=rng.normal(size=(nr, n)) * 0.3)
    E = np.linspace(-2.5, 2.5, 11)
    r = transport_tdb(E, blocks, eta=0.0, eta0=1e-4, convergence=1e-13, dev_factor=1.0,
                      precision="mixed", refine_iters=2)
    o = N.transport(E, blocks, 0.0, 1e-4, 1e-13, 1.0)
    assert (r["status"] == 0).all()
    assert np.abs(r["transl"] - o["transl"]).max() < 1e-8 * max(1.0, np.abs(o["transl"]).max())
    assert np.abs(r["iters"][:, 0] - o["iters_left"]).max() <= 1


@pytest.mark.parametrize("precision,ne", [("fp64", 96), ("mixed", 96), ("mixed", 300)])
def test_graph_replay_matches_direct_run(cuda_ready, precision, ne):
    """The batched pass captured into a CUDA graph and replayed gives the
    direct run's T bit for bit (same kernels, same order); with 300 points
    the mixed path splits the batch over two streams, which the capture
    records as a fork and a join."""
    import torch
    from phinfortran_gb300 import DeviceTransport
    b, E, p = S.tb_ribbon(W=24, L=40, ne=ne)
    Ed = torch.from_numpy(E).cuda()
    dt = DeviceTransport(b, E.size, precision=precision, **p)
    dt.run(Ed)
    torch.cuda.synchronize()
    T0 = dt.transl[:E.size].cpu().numpy().copy()
    g = dt.capture(Ed)
    dt.transl.zero_()
    for _ in range(2):
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(dt.transl[:E.size].cpu().numpy(), T0)
        assert (dt.status[:E.size].cpu().numpy() == 0).all()


def test_lead_arithmetics_on_the_ribbon(cuda_ready):
    """The default mixed path (FP64-grade lead decimations with their block
    products on the tensor cores, FP32 factorisation, double-float
    refinement) against the FP64 path on 512 energies of the disordered
    32-wide ribbon (L = 100, eta = 1e-6): every point where FP64 itself is
    reproducible (a 1e-15 relative perturbation of the blocks moves its T by
    at most 1e-10) within 1e-8 relative (|T - T64| / max(|T64|, 1e-3)).  The
    faster lead arithmetics (split: first 8 steps FP64; all double-float)
    keep the median but not the maximum."""
    import torch
    from phinfortran_gb300 import DeviceTransport
    b, E, p = S.tb_ribbon(W=32, L=100, ne=512)
    Ed = torch.from_numpy(E).cuda()
    f64 = DeviceTransport(b, E.size, precision="fp64", **p)
    f64.run(Ed)
    torch.cuda.synchronize()
    T64 = f64.transl[:E.size].cpu().numpy().copy()
    rng = np.random.default_rng(123)
    bp = {k: np.asarray(v) * (1 + 1e-15 * rng.standard_normal(np.shape(v))) for k, v in b.items()}
    fp = DeviceTransport(bp, E.size, precision="fp64", **p)
    fp.run(Ed)
    torch.cuda.synchronize()
    good = rel(fp.transl[:E.size].cpu().numpy(), T64) <= 1e-10
    assert good.mean() > 0.7
    out = {}
    for lead in ("auto", "fp64", "split", "df64"):
        dt = DeviceTransport(b, E.size, precision="mixed", lead_arith=lead, **p)
        dt.run(Ed)
        torch.cuda.synchronize()
        assert (dt.status[:E.size].cpu().numpy() == 0).all()
        out[lead] = rel(dt.transl[:E.size].cpu().numpy(), T64)
    # blocks of 32: the default is the FP64 tensor-core decimation
    assert np.array_equal(out["auto"], out["fp64"])
    r = out["fp64"]
    assert r[good].max() <= 1e-8, (r[good].max(), int(np.argmax(np.where(good, r, 0))))
    assert np.median(r) < 1e-9
    for lead in ("split", "df64"):
        assert np.median(out[lead]) < 1e-9, lead
        assert out[lead].max() < 1e-2, lead
