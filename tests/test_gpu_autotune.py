"""The large-block autotuner: it times the caller's problem for each
(panel width, batch) candidate, keeps the fastest, caches it per shape, and
the tuned engine gives the FP64 result of the built-in choice (panel width
changes only the rounding order of the blocked inverse)."""
import json

import numpy as np
import pytest

from phinfortran_gb300 import systems as S
from phinfortran_gb300 import transport_tdb
from phinfortran_gb300.autotune import apply_tuning, autotune_tiled, layout, set_tuning

pytestmark = pytest.mark.gpu


def test_autotune_diamond_n216(cuda_ready, tmp_path):
    b, E, p, aux = S.diamond_phonon(nc=3, L=4, kpoints=[0])
    bq = {k: v[0] for k, v in b.items()}
    Es = E[np.linspace(10, 500, 6).astype(int)]
    cache = str(tmp_path / "tune.json")
    try:
        set_tuning(0, 0)
        ref = transport_tdb(Es, bq, want_transr=False, precision="tc", **p)["transl"]
        best = autotune_tiled(Es, bq, precision="tc", panels=(8, 32), batches=(4, 256), cache=cache, **p)
        assert best["seconds"] <= best["default_seconds"]
        assert len(best["candidates"]) >= 2
        table = json.load(open(cache))
        assert len(table) == 1 and list(table.values())[0]["panel"] == best["panel"]
        got = apply_tuning(bq, precision="tc", cache=cache)
        assert got["batch"] == best["batch"]
        r = transport_tdb(Es, bq, want_transr=False, precision="tc", **p)["transl"]
        assert np.abs(r - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())
        set_tuning(8, 4)
        assert layout(216, 216, 216, 6, "tc") == (8, 4)
    finally:
        set_tuning(0, 0)
