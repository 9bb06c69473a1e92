"""GPU D(q) block assembly (pf_gen_dyn_qe_tdb) against the oracle's
restatement of gen_dyn_qe_tdb_k and, through the transport kernel, against
the reference's committed si-si transmissions."""
import numpy as np
import pytest

from phinfortran_gb300 import transport_tdb
from phinfortran_gb300.dyn import gen_dyn_qe_tdb
from tests.sisi_case import golden_close, sisi_blocks, sisi_params

pytestmark = pytest.mark.gpu


def _geom(f):
    nb = f["n_bloch"]
    return dict(fc=f["fc"], cell=f["cell"], pos=f["pos"], cell_all=f["cell_all"], pos_all=f["pos_all"],
                idxall=f["idxall"], mass_all=f["mass_all"], rws=f["rws"], rd=f["rd"],
                n_bloch_x=int(nb[0]), n_bloch_y=int(nb[1]), buffer_left=int(f["buffer"]),
                period_left=int(f["period"]), buffer_right=int(f["buffer"]), period_right=int(f["period"]),
                nlayer=int(f["nlayer"]), natm_layer=int(f["natm_layer"]))


def test_assembly_matches_oracle(cuda_ready, sisi):
    ks = [0, 3, 17, 24, 48]
    g = gen_dyn_qe_tdb(sisi["kgrid"][ks], **_geom(sisi))
    for i, k in enumerate(ks):
        o = sisi_blocks(sisi, k)
        for name in o:
            ref = np.asarray(o[name])
            got = g[name][i]
            assert got.shape == ref.shape, name
            scale = max(np.abs(ref).max(), 1.0)
            assert np.abs(got - ref).max() <= 1e-13 * scale, (name, k, np.abs(got - ref).max())


def test_assembly_feeds_transport_all_k(cuda_ready, sisi):
    """GPU-assembled blocks for all 49 k -> one transport launch -> golden T."""
    g = gen_dyn_qe_tdb(sisi["kgrid"], **_geom(sisi))
    E1 = sisi["E"]
    nk = 49
    E = np.tile(E1, nk)
    q = np.repeat(np.arange(nk), E1.size).astype(np.int32)
    zf = np.zeros(E.size, np.int32)
    zf[::E1.size] = 1
    r = transport_tdb(E, g, qidx=q, zero_flag=zf, want_transr=True, **sisi_params(sisi))
    TL = r["transl"].reshape(nk, E1.size).T
    ok, ad, q99 = golden_close(TL, sisi["transl_tot"])
    assert ok, (ad, q99)
