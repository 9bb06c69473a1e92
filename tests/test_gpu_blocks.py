"""Green's-function blocks of pf_transport_tdb_blocks_dev (what the
reference's vel_mat_tdb receives from surface_green_tdb_mpi and
get_G_full_tdb_mpi) against the oracle: the four surface functions, the two
broadenings, G_{0,N+1}, G_{N+1,0}, G_L and G_R, on the si-si leads (nl = nr,
the identical-lead shortcut) and on a system with uneven lead and device
widths.  Every call goes through the C ABI."""
import numpy as np
import pytest

from oracle import negf as N
from phinfortran_gb300.modes import BLOCK_OUTPUTS, transport_tdb_blocks
from tests.sisi_case import sisi_blocks, sisi_params

pytestmark = pytest.mark.gpu

SURFACE = ("gl_adv", "gl_plus", "gr_ret", "gr_minus", "gml_adv", "gmr_ret")
DEVICE = ("G_D_LR", "G_R", "G_D_RL", "G_L")


def _blockwise_rel(a, b, scale=None):
    """Per point: max |a - b| over the block / max |scale| (default b) over the block."""
    d = np.abs(a - b).reshape(a.shape[0], -1).max(axis=1)
    ref = b if scale is None else scale
    s = np.abs(ref).reshape(ref.shape[0], -1).max(axis=1)
    return d / np.maximum(s, 1e-300)


# the broadenings i (Sigma - Sigma^H) are differences: their rounding is
# relative to the self-energy, which can be much larger near a band bottom
SCALE = dict(gml_adv="sl_adv", gmr_ret="sr_ret")


def _check(r, o, tol):
    for k in SURFACE:
        sc = o["surface"][SCALE[k]] if k in SCALE else None
        e = _blockwise_rel(r[k], o["surface"][k], sc)
        assert e.max() < tol, (k, float(e.max()))
    for k in DEVICE:
        e = _blockwise_rel(r[k], o[k])
        assert e.max() < tol, (k, float(e.max()))
    assert np.abs(r["transl"] - o["transl"]).max() <= tol * max(1.0, np.abs(o["transl"]).max())


def test_blocks_sisi(cuda_ready, sisi):
    b = sisi_blocks(sisi, 3)
    p = sisi_params(sisi)
    E = sisi["E"][1::6]
    r = transport_tdb_blocks(E, b, **p)
    o = N.transport(E, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"], want_blocks=True,
                    want_plus_minus=True)
    assert (r["status"] == 0).all()
    _check(r, o, 1e-8)


def test_blocks_uneven_widths_and_subset(cuda_ready):
    rng = np.random.default_rng(9)
    n, nl, nr, L = 7, 4, 5, 3

    def herm(m):
        a = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
        return a + a.conj().T

    blocks = dict(HL=herm(nl), HLv=rng.normal(size=(nl, nl)) * 0.5, HR=herm(nr),
                  HRv=rng.normal(size=(nr, nr)) * 0.5, Hd=np.stack([herm(n) for _ in range(L)]),
                  Hdv=rng.normal(size=(L - 1, n, n)) * 0.5, Hld=rng.normal(size=(nl, n)) * 0.5,
                  Hrd=rng.normal(size=(nr, n)) * 0.5)
    E = np.linspace(-3, 3, 9)
    kw = dict(eta=0.0, eta0=1e-3, convergence=1e-12, dev_factor=1.0)
    r = transport_tdb_blocks(E, blocks, **kw)
    o = N.transport(E, blocks, 0.0, 1e-3, 1e-12, 1.0, want_blocks=True, want_plus_minus=True)
    assert r["G_D_LR"].shape == (E.size, nl, nr) and r["G_D_RL"].shape == (E.size, nr, nl)
    _check(r, o, 1e-9)
    # a subset: only the requested blocks come back, T is unchanged
    s = transport_tdb_blocks(E, blocks, want=("G_D_LR",), **kw)
    assert set(s) == {"transl", "transr", "status", "G_D_LR"}
    assert np.array_equal(s["G_D_LR"], r["G_D_LR"])
    assert np.array_equal(s["transl"], r["transl"])
    assert set(BLOCK_OUTPUTS) == set(SURFACE) | set(DEVICE)
