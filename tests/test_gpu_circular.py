"""Block-circulant leads on the GPU (pf_transport_tdb_tiled_circ_dev,
circular_flag = 1) against the oracle's restatement of circular_g
(negf/circular.f90:42-105; oracle/circular.py).

* si-si leads (2 x 2 Bloch supercell, n_l = 48, G.R = 2 pi): T_L within
  1e-9 relative of the oracle's circular path and of the FP64 direct
  decimation.
* diamond slabs at the transverse Gamma point (nc x nc cells: block
  circulant with nc outer and nc inner blocks of 24): n = 96 and 216, with
  the FP64, tensor-core and double-float block arithmetics.
* leads whose rows below the first block row are perturbed: circular_g
  reads only the first block rows, so the GPU must follow the oracle's
  circular result, which then differs from the direct decimation."""
import numpy as np
import pytest

from oracle import circular as C
from oracle import negf as N
from phinfortran_gb300 import systems as S
from phinfortran_gb300 import transport_tdb
from tests.sisi_case import sisi_blocks, sisi_params

pytestmark = pytest.mark.gpu

TWO_PI = 2.0 * np.pi


@pytest.fixture(scope="module")
def fx():
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    return np.load(os.path.join(here, "golden", "sisi.npz"))


def _sisi_gr(fx):
    cell = np.asarray(fx["cell"], dtype=np.float64)
    reci = 2.0 * np.pi * np.linalg.inv(cell).T
    return [float(reci[1] @ cell[1]), float(reci[0] @ cell[0])] * 2


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)) / np.maximum(np.abs(np.asarray(b)), 1.0)


@pytest.mark.parametrize("ik", [5, 24])
def test_circular_sisi(cuda_ready, fx, ik):
    p = sisi_params(fx)
    b = {k: np.asarray(v) for k, v in sisi_blocks(fx, ik).items()}
    E = np.asarray(fx["E"][1:60:5], dtype=np.float64)
    gr = _sisi_gr(fx)
    r = transport_tdb(E, b, want_transr=False, circular=(2, 2, gr), **p)
    assert (r["status"] == 0).all()
    To = C.transport_circular(E, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"], 2, 2, gr)
    Td = transport_tdb(E, b, want_transr=False, **p)["transl"]
    assert _rel(r["transl"], To).max() < 1e-9
    assert _rel(r["transl"], Td).max() < 1e-9
    assert (r["iters"] > 0).all()


@pytest.mark.parametrize("nc,cells,precision,tol", [(2, (2, 2), "fp64", 1e-9), (3, (3, 3), "fp64", 1e-9),
                                                    (3, (3, 3), "tc", 1e-9), (2, (2, 2), "df64", 1e-6),
                                                    (3, (3, 1), "fp64", 1e-9)])
def test_circular_diamond_gamma(cuda_ready, nc, cells, precision, tol):
    """Small blocks of 24 (resident decimation, one CTA a block; batched
    double-float engine for df64) and, with 3 x 1 cells, of 72 (batched
    small-block engine)."""
    b, E, p, aux = S.diamond_phonon(nc=nc, L=6, nk_side=1, ne=12)
    bq = {k: v[0] for k, v in b.items()}
    E = E[1::2]
    ny, nx = cells
    r = transport_tdb(E, bq, want_transr=False, circular=(ny, nx, [TWO_PI] * 4), precision=precision, **p)
    assert (r["status"] == 0).all()
    To = C.transport_circular(E, bq, p["eta"], p["eta0"], p["convergence"], p["dev_factor"], ny, nx,
                              [TWO_PI] * 4)
    assert To.max() > 1.0
    assert _rel(r["transl"], To).max() < tol, _rel(r["transl"], To).max()


def test_circular_sisi_two_q(cuda_ready, fx):
    """Two k block sets interleaved in one call (qidx): every q batch is
    transformed with its own lead matrices."""
    p = sisi_params(fx)
    bs = [{k: np.asarray(v) for k, v in sisi_blocks(fx, ik).items()} for ik in (3, 40)]
    st = {k: np.stack([bs[0][k], bs[1][k]]) for k in bs[0]}
    E1 = np.asarray(fx["E"][2:60:7], dtype=np.float64)
    E = np.repeat(E1, 2)
    q = np.tile(np.array([0, 1], dtype=np.int32), E1.size)
    gr = _sisi_gr(fx)
    r = transport_tdb(E, st, qidx=q, want_transr=False, circular=(2, 2, gr), **p)
    assert (r["status"] == 0).all()
    for qq in (0, 1):
        sel = q == qq
        To = C.transport_circular(E[sel], bs[qq], p["eta"], p["eta0"], p["convergence"], p["dev_factor"], 2, 2, gr)
        assert _rel(r["transl"][sel], To).max() < 1e-9


def test_circular_reads_first_block_rows(cuda_ready, fx):
    """Rows of H_L below the first block row perturbed: the direct
    decimation changes, circular_g does not (it transforms the first block
    row only), and the GPU follows circular_g."""
    p = sisi_params(fx)
    b = {k: np.asarray(v).copy() for k, v in sisi_blocks(fx, 5).items()}
    rng = np.random.default_rng(3)
    n = b["HL"].shape[0]
    pert = np.zeros((n, n), np.complex128)
    x = 0.02 * np.abs(b["HL"]).max() * rng.standard_normal((n - n // 2, n - n // 2))
    pert[n // 2:, n // 2:] = x + x.T   # hermitian, outside the first block row
    b["HL"] = b["HL"] + pert
    E = np.asarray(fx["E"][10:50:8], dtype=np.float64)
    gr = _sisi_gr(fx)
    r = transport_tdb(E, b, want_transr=False, circular=(2, 2, gr), check=False, **p)
    To = C.transport_circular(E, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"], 2, 2, gr)
    Tdir = N.transport(E, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"], max_iter=1000)["transl"]
    assert _rel(Tdir, To).max() > 1e-6
    assert _rel(r["transl"], To).max() < 1e-9


def test_circular_rejects_bad_cells(cuda_ready, fx):
    p = sisi_params(fx)
    b = {k: np.asarray(v) for k, v in sisi_blocks(fx, 0).items()}
    with pytest.raises(ValueError):
        transport_tdb(np.array([0.1]), b, want_transr=False, circular=(5, 2, [TWO_PI] * 4), **p)


def test_circular_transr(cuda_ready, fx):
    """T_R with block-circulant leads: the right-to-left sweep after the
    circular surface functions, against the oracle's direct T_R."""
    p = sisi_params(fx)
    b = {k: np.asarray(v) for k, v in sisi_blocks(fx, 24).items()}
    E = np.asarray(fx["E"][3:60:9], dtype=np.float64)
    r = transport_tdb(E, b, want_transr=True, circular=(2, 2, _sisi_gr(fx)), **p)
    assert (r["status"] == 0).all()
    o = N.transport(E, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"])
    assert _rel(r["transr"], o["transr"]).max() < 1e-9
    assert _rel(r["transl"], o["transl"]).max() < 1e-9
