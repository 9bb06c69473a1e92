"""The C restatement of the transmission oracle (oracle/negf_c.c, the CPU
baseline of bench.py) against the numpy oracle and the reference's si-si
output (CPU)."""
import numpy as np

from oracle import negf as N
from oracle.negf_c import transport_c
from phinfortran_gb300 import systems as S
from tests.sisi_case import golden_close, sisi_blocks, sisi_params


def test_c_oracle_matches_numpy_oracle():
    for b, E, p in (S.tb_ribbon(W=8, L=12, ne=24), S.sc_phonon(ne=32)[:3]):
        o = N.transport(E, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"])
        T, it, used = transport_c(E, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"], threads=2)
        assert used >= 1
        assert np.array_equal(it, o["iters_left"])
        rel = np.abs(T - o["transl"]) / np.maximum(np.abs(o["transl"]), 1e-3)
        assert np.median(rel) < 1e-11 and rel.max() < 1e-6, rel.max()


def test_c_oracle_matches_reference_output(sisi):
    ik = 10
    b = sisi_blocks(sisi, ik)
    p = sisi_params(sisi)
    T, _, _ = transport_c(sisi["E"], b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"])
    T[0] = 0.0                                     # the ie == 1 rule
    ok, ad, q99 = golden_close(T, sisi["transl_tot"][:, ik], abs_tol=1e-6, rel_q99=1e-8)
    assert ok, (ad, q99)
