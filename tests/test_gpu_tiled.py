"""Large-block FP64 path (pf_transport_tdb_tiled_dev) against the oracle:
blocks above the resident limit (48), both the shared-memory inverse and the
blocked Gauss-Jordan inverse (ragged last panel), several q block sets."""
import numpy as np
import pytest

from oracle import negf as N
from phinfortran_gb300 import systems as S
from phinfortran_gb300 import transport_tdb

pytestmark = pytest.mark.gpu


def check_against_oracle(b, E, p, qidx=None, zf=None, tol=1e-9, precision="fp64"):
    r = transport_tdb(E, b, want_transr=False, qidx=qidx, zero_flag=zf, precision=precision, **p)
    assert (r["status"] == 0).all()
    if qidx is None:
        o = N.transport(E, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"],
                        zero_first=None if zf is None else zf.astype(bool))
        To, it = o["transl"], o["iters_left"]
    else:
        To = np.zeros(E.size)
        it = np.zeros(E.size, dtype=int)
        for q in np.unique(qidx):
            sel = qidx == q
            bq = {k: v[q] for k, v in b.items()}
            o = N.transport(E[sel], bq, p["eta"], p["eta0"], p["convergence"], p["dev_factor"])
            To[sel] = o["transl"]
            it[sel] = o["iters_left"]
    err = np.abs(r["transl"] - To) / np.maximum(np.abs(To), 1.0)
    assert err.max() < tol, (err.max(), np.argmax(err))
    # same stopping rule as the oracle's decimation
    assert np.abs(r["iters"][:, 0] - it).max() <= 1
    return r, To


def test_tiled_small_inverse(cuda_ready):
    """6 x 6 cross-section: n = 108 (shared-memory inverse)."""
    b, E, p, _ = S.sc_phonon(nx=6, ny=6, L=5, ne=20, seed_index=11)
    zf = np.zeros(E.size, np.int32)
    zf[0] = 1
    r, o = check_against_oracle(b, E, p, zf=zf)
    assert r["transl"][0] == 0.0
    assert o.max() > 1.0


def test_tiled_blocked_inverse(cuda_ready):
    """7 x 7 cross-section: n = 147 -> blocked Gauss-Jordan, panels of 32
    and a last panel of 19 columns."""
    b, E, p, _ = S.sc_phonon(nx=7, ny=7, L=3, ne=10, seed_index=12)
    check_against_oracle(b, E[1:], p)


def test_tiled_multi_q(cuda_ready):
    """Two block sets (different disorder seeds) interleaved in one call."""
    b1, E, p, _ = S.sc_phonon(nx=6, ny=6, L=4, ne=12, seed_index=13)
    b2, _, _, _ = S.sc_phonon(nx=6, ny=6, L=4, ne=12, seed_index=14)
    st = {k: np.stack([b1[k], b2[k]]) for k in b1}
    Eint = np.repeat(E[1:], 2)
    q = np.tile(np.array([0, 1], dtype=np.int32), E.size - 1)
    check_against_oracle(st, Eint, p, qidx=q)


def test_tiled_diamond_slab_interface(cuda_ready):
    """Diamond slab stack (2 x 2 conventional cells, n = 96) with a 28 / 72.6
    mass interface: different left and right leads, two transverse k."""
    b, E, p, aux = S.diamond_phonon(nc=2, L=6, nk_side=8, ne=24, kpoints=[5, 27], block=3)
    Es = E[2:22:3]
    q = np.repeat(np.arange(2, dtype=np.int32), Es.size)
    check_against_oracle(b, np.tile(Es, 2), p, qidx=q)


def test_tiled_diamond_blocked(cuda_ready):
    """3 x 3 cells: n = 216, blocked inverse (six panels of 32, one of 24)."""
    b, E, p, aux = S.diamond_phonon(nc=3, L=3, nk_side=8, ne=12, kpoints=[9], block=2)
    bq = {k: v[0] for k, v in b.items()}
    check_against_oracle(bq, E[3:9:2], p)


@pytest.mark.parametrize("nc,kp", [(2, 27), (3, 9)])
def test_tiled_double_float(cuda_ready, nc, kp):
    """precision="df64" above 48: the tiled engine in double-float
    arithmetic (FP32 pipe); T within 1e-8 of the FP64 oracle (n = 96 and the
    blocked inverse at n = 216)."""
    b, E, p, aux = S.diamond_phonon(nc=nc, L=4, nk_side=8, ne=12, kpoints=[kp], block=2)
    bq = {k: v[0] for k, v in b.items()}
    check_against_oracle(bq, E[2:11:2], p, tol=1e-8, precision="df64")


@pytest.mark.parametrize("case", ["sc108", "sc147", "diamond96", "diamond216"])
def test_tiled_tensor_core(cuda_ready, case):
    """precision="tc": the FP64 algorithm with every block product on the
    tcgen05 tensor cores (exact BF16 slice products assembled in FP64); the
    FP64 oracle's T within 1e-9 and its decimation counts within 1, for the
    shared-memory inverse (n = 96, 108) and the blocked inverse whose
    trailing updates are tensor-core products (n = 147, 216)."""
    if case == "sc108":
        b, E, p, _ = S.sc_phonon(nx=6, ny=6, L=5, ne=20, seed_index=11)
        check_against_oracle(b, E[1:], p, precision="tc")
    elif case == "sc147":
        b, E, p, _ = S.sc_phonon(nx=7, ny=7, L=3, ne=10, seed_index=12)
        check_against_oracle(b, E[1:], p, precision="tc")
    elif case == "diamond96":
        b, E, p, aux = S.diamond_phonon(nc=2, L=6, nk_side=8, ne=24, kpoints=[5, 27], block=3)
        Es = E[2:22:3]
        q = np.repeat(np.arange(2, dtype=np.int32), Es.size)
        check_against_oracle(b, np.tile(Es, 2), p, qidx=q, precision="tc")
    else:
        b, E, p, aux = S.diamond_phonon(nc=3, L=3, nk_side=8, ne=12, kpoints=[9], block=2)
        bq = {k: v[0] for k, v in b.items()}
        check_against_oracle(bq, E[3:9:2], p, precision="tc")


@pytest.mark.parametrize("system,precision", [("bar", "fp64"), ("bar", "tc"), ("diamond", "fp64"),
                                              ("diamond", "tc")])
def test_tiled_transr(cuda_ready, system, precision):
    """want_transr on the large-block engine (pf_transport_tdb_tiled_ex_dev):
    the right-to-left sweep and T_R (negf/lesser.f90:694-800) against the
    oracle's, on a disordered bar (n = 108, identical leads: the right
    surface function mirrored from the left) and on a diamond slab with a
    mass interface (n = 96, leads of different mass: both decimated), and
    T_L unchanged by the option."""
    if system == "bar":
        b, E, p, _ = S.sc_phonon(nx=6, ny=6, L=5, ne=16, seed_index=15, lead_mass=1.3)
        E = E[1:]
    else:
        bq, E, p, _ = S.diamond_phonon(nc=2, L=6, nk_side=1, ne=16, block=3)
        b = {k: v[0] for k, v in bq.items()}
        E = E[1::2]
        assert not np.array_equal(b["HL"], b["HR"])
    r = transport_tdb(E, b, want_transr=True, precision=precision, **p)
    assert (r["status"] == 0).all()
    o = N.transport(E, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"])
    rel = lambda a, c: np.abs(a - c) / np.maximum(np.abs(c), 1.0)
    assert rel(r["transr"], o["transr"]).max() < 1e-9
    assert rel(r["transl"], o["transl"]).max() < 1e-9
    r0 = transport_tdb(E, b, want_transr=False, precision=precision, **p)
    assert np.array_equal(r0["transl"], r["transl"])
