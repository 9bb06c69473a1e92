"""GPU tight-binding blocks (pf_tb_hk_blocks) against the oracle's dense
gen_ham H(k) (oracle/tb.py), for a two-species structure with s, p, d and
s* orbitals, and the block set fed to the transport entry."""
import numpy as np
import pytest

from oracle import negf as N
from oracle import tb as TB
from phinfortran_gb300 import transport_tdb
from phinfortran_gb300.tb import tb_blocks, tdb_from_layers

pytestmark = pytest.mark.gpu

ORBS = [["s", "px", "py", "pz", "s*"], ["s", "dxy", "dyz", "dxz", "dx2-y2", "dz2", "px"]]


def structure(nlayers=6, seed=3, jitter_all=True):
    """Layers of three atoms (two species) along z, 2.2 A apart, jittered
    (only the inner layers unless jitter_all: the two outer layers on each
    side then form periodic leads); transverse cell 5 A x 5 A.  Units as the
    reference holds them: positions in Angstrom, r_d in metres (V_term scales
    by (r_d / |r| / 1e-10)^Vn)."""
    rng = np.random.default_rng(seed)
    A = 1.0
    base = np.array([[0.0, 0.0, 0.0], [2.5, 0.3, 0.4], [1.1, 2.6, 0.9]]) * A
    pos, spec = [], []
    for L in range(nlayers):
        for i, b in enumerate(base):
            jit = rng.uniform(-0.15, 0.15, 3) * A
            if not jitter_all and (L < 2 or L >= nlayers - 2):
                jit = 0.0
            pos.append(b + np.array([0, 0, 2.2 * L]) * A + jit)
            spec.append(i % 2)
    lat = np.array([[5.0, 0, 0], [0, 5.0, 0], [0, 0, 2.2 * nlayers + 30.0]]) * A
    rng2 = np.random.default_rng(seed + 1)
    V = rng2.uniform(-2, 2, size=(2, 2, 4, 4, 4))
    Vn = rng2.uniform(1.0, 3.0, size=(2, 2, 4, 4, 4))
    r_d = np.array([[2.35, 2.4], [2.4, 2.45]]) * 1e-10
    blk = np.arange(0, 3 * nlayers + 1, 3)
    return np.array(pos), np.array(spec), V, Vn, r_d, lat, blk


def test_tb_blocks_match_oracle(cuda_ready):
    pos, spec, V, Vn, r_d, lat, blk = structure()
    kf = np.array([[0.0, 0.0, 0.0], [0.21, -0.37, 0.0], [0.5, 0.5, 0.0]])
    diag, upper = tb_blocks(pos, spec, ORBS, V, Vn, r_d, lat, 3.1, kf, blk)
    rec = 2 * np.pi * np.linalg.inv(lat).T
    codes = [[TB.NAMES.index(o) for o in lst] for lst in ORBS]
    rows = TB.orbital_list(spec, codes)
    first = np.concatenate([[0], np.cumsum([len(codes[s]) for s in spec])])
    for k in range(kf.shape[0]):
        H = TB.gen_ham(pos, spec, codes, V, Vn, r_d, lat, 3.1, kf[k], rec)
        scale = np.abs(H).max()
        for I in range(len(blk) - 1):
            a0, a1 = first[blk[I]], first[blk[I + 1]]
            assert np.abs(diag[k][I] - H[a0:a1, a0:a1]).max() < 1e-12 * scale
            if I + 2 < len(blk):
                b1 = first[blk[I + 2]]
                assert np.abs(upper[k][I] - H[a0:a1, a1:b1]).max() < 1e-12 * scale
    assert len(rows) == first[-1]


def test_tb_blocks_feed_transport(cuda_ready):
    """Layers [lead -1, lead 0, device 1..2, lead N+1, lead N+2] of the same
    structure: T through the transport entry equals the oracle's T on the
    same blocks (electron conventions: dev_factor 1, eta = 0)."""
    pos, spec, V, Vn, r_d, lat, blk = structure(nlayers=7, jitter_all=False)
    kf = np.array([[0.1, 0.2, 0.0]])
    diag, upper = tb_blocks(pos, spec, ORBS, V, Vn, r_d, lat, 3.1, kf, blk)
    b = tdb_from_layers(diag[0], upper[0])
    p = dict(eta=0.0, eta0=1e-4, convergence=1e-12, dev_factor=1.0)
    E = np.linspace(-1.0, 1.0, 7)
    r = transport_tdb(E, b, want_transr=False, max_iter=2000, **p)
    o = N.transport(E, b, max_iter=2000, **p)
    np.testing.assert_allclose(r["transl"], o["transl"], rtol=1e-8, atol=1e-10)
