"""GPU Landauer conductance against the condt.py restatement on the reference's si-si output."""
import numpy as np
import pytest

from oracle import post
from phinfortran_gb300.conductance import conductance

pytestmark = pytest.mark.gpu

AREA = (5.46616 * np.sqrt(2)) ** 2 * 1.0e-20   # condt.py:8


def test_conductance_sisi(cuda_ready, sisi):
    E = sisi["E_transr_tot"]
    tr = sisi["transr_tot"]
    temps = np.linspace(10, 700, 100)              # condt.py:56
    got = conductance(E, tr, temps, AREA)
    w = post.omega_from_egrid(E)
    ref = np.array([post.condt(w, t, tr.sum(axis=1) / tr.shape[1], AREA) for t in temps])
    np.testing.assert_allclose(got, ref, rtol=1e-12)
    assert (got > 0).all()
