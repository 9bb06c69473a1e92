"""Block-circulant surface Green's function (circular_flag = 1).

The reference can replace each lead decimation by circular_g
(negf/circular.f90:42-105): Fourier-transform the lead matrices of the
n_bloch_y x n_bloch_x supercell to block-diagonal form, decimate every small
block, transform back.  The engines here always decimate the full lead
matrices; this test restates circular_g (oracle/circular.py) and checks on
the si-si leads (2 x 2 Bloch supercell, n_l = 48) that both give the same
surface Green's function for all four decimations of surface_green_tdb
(negf/surface.f90:486-590), at several k and energies, so a run with
circular_flag = 1 is reproduced by the direct decimation."""
import numpy as np
import pytest

from oracle import circular as C
from tests.sisi_case import sisi_blocks, sisi_params


@pytest.fixture(scope="module")
def fx():
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    return np.load(os.path.join(here, "golden", "sisi.npz"))


@pytest.mark.parametrize("ik,ie", [(0, 7), (5, 20), (24, 41), (40, 58)])
def test_circular_equals_direct(fx, ik, ie):
    b = sisi_blocks(fx, ik)
    p = sisi_params(fx)
    cell = np.asarray(fx["cell"], dtype=np.float64)
    reci = 2.0 * np.pi * np.linalg.inv(cell).T
    n = b["HL"].shape[0]
    P1 = C.set_pmatrix(n, 2, reci[1], cell[1])          # negf/phinfortran.f90:622-628, left lead
    P2 = C.set_pmatrix(n // 2, 2, reci[0], cell[0])
    E = float(fx["E"][ie])
    eps = E * p["eta"] + p["eta0"]
    cases = [(E - 1j * eps, b["HL"], b["HLv"].conj().T),      # left advanced   (surface.f90:484-504)
             (E + 1j * eps, b["HL"], b["HLv"]),               # left "plus"     (:510-535)
             (E + 1j * eps, b["HR"], b["HRv"].conj().T),      # right retarded  (:540-565)
             (E - 1j * eps, b["HR"], b["HRv"])]               # right "minus"   (:571-596)
    for z, h00, alpha in cases:
        Es0 = z * np.eye(n)
        g = C.decimation(Es0, h00, alpha, p["convergence"])
        gc = C.circular_g(Es0, h00, alpha, alpha.conj().T, p["convergence"], n, 2, 2, reci[1], cell[1],
                          reci[0], cell[0], P1=P1, P2=P2)
        assert np.abs(gc - g).max() <= 1e-10 * np.abs(g).max()
