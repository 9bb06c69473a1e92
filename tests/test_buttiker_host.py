"""Buttiker probes (oracle/buttiker.py, restating negf/lesser.f90:12-45,
475-680, 1199-1623): the probe-aware G_full and the lesser function of the
recursion against a dense solution of the same device (lead self-energies
folded in, probe self-energies on the diagonal, Gn = G Sigma_in G^H), the
Jacobian against central differences of the fluxes in the probe
temperatures, and the host Newton pieces of the package against the oracle.
The reference ships no Buttiker example, so the path is checked for
internal consistency; parity with the reference is unpinned."""
import numpy as np
import pytest

from oracle import buttiker as BP
from oracle import negf as N
from phinfortran_gb300 import buttiker as PB
from phinfortran_gb300 import systems as S

H = N.H
B_PROBE = 5.0e-20 * (2.0 * 3.1415926 * 1.0e12) * 1.0e3


@pytest.fixture(scope="module")
def bar():
    b, E, p, aux = S.sc_phonon(nx=2, ny=2, L=5, ne=33, mass_range=(1.0, 2.0))
    return b, E, p


def _leads(b, E, p):
    s = N.surface_green_tdb(E, b["HL"], b["HLv"], b["HR"], b["HRv"], p["eta"], p["eta0"], p["convergence"],
                            want_plus_minus=False)
    return H(s["gl_adv"]), s["gr_ret"], -s["gml_adv"], s["gmr_ret"], s["sr_ret"]


def test_recursion_equals_dense_solution(bar):
    b, E, p = bar
    L, n = b["Hd"].shape[0], b["Hd"].shape[-1]
    Eg = np.array([E[6], E[17]])
    temps = BP.initial_temperatures(L, 300.0, 310.0)
    sw, dsw = BP.set_sigma_bp_w(temps, Eg, B_PROBE, 430.0)
    gl, gr, gml, gmr, sr = _leads(b, Eg, p)
    g = BP.g_full_probes(Eg, gl, gr, gml, gmr, sr, b["Hd"], b["Hdv"], b["Hld"], b["Hrd"], b["HR"], sw.T,
                         p["eta"], p["eta0"], 10.0)
    r = BP.g_lesser(Eg, np.zeros(2, bool), gl, gr, g["GLeft"], g["G_full"], g["G_q_qp"], b["Hdv"], b["Hld"],
                    b["Hrd"], sw.T, dsw.T, temps, 300.0, 310.0)
    for k in range(2):
        zD = Eg[k] + 1j * 10.0 * (Eg[k] * p["eta"] + p["eta0"])
        A = np.zeros((L * n, L * n), complex)
        for i in range(L):
            A[i * n:(i + 1) * n, i * n:(i + 1) * n] = zD * np.eye(n) - b["Hd"][i] - sw[i, k] * np.eye(n)
            if i < L - 1:
                A[i * n:(i + 1) * n, (i + 1) * n:(i + 2) * n] = -b["Hdv"][i]
                A[(i + 1) * n:(i + 2) * n, i * n:(i + 1) * n] = -H(b["Hdv"][i])
        SL = H(b["Hld"]) @ gl[k] @ b["Hld"]
        V1 = H(b["Hrd"])
        SR = V1 @ gr[k] @ H(V1)
        A[:n, :n] -= SL
        A[-n:, -n:] -= SR
        G = np.linalg.inv(A)
        fr = np.sqrt(Eg[k])
        f = [BP.bose_einstein(fr, T) for T in temps]
        Sin = np.zeros_like(A)
        for i in range(L):
            Sin[i * n:(i + 1) * n, i * n:(i + 1) * n] = 1j * (sw[i, k] - np.conj(sw[i, k])) * f[i] * np.eye(n)
        Sin[:n, :n] += 1j * (SL - H(SL)) * BP.bose_einstein(fr, 300.0)
        Sin[-n:, -n:] += 1j * (SR - H(SR)) * BP.bose_einstein(fr, 310.0)
        Gn = G @ Sin @ H(G)
        for i in range(L):
            s = slice(i * n, (i + 1) * n)
            assert np.abs(G[s, s] - g["G_full"][k, i]).max() < 1e-12 * np.abs(G).max()
            assert abs(np.trace(Gn[s, s]) - r["Gn_i"][k, i]) < 1e-10 * abs(np.trace(Gn[s, s]))


def test_jacobian_matches_finite_differences(bar):
    b, E, p = bar
    L = b["Hd"].shape[0]
    Eg = np.array([E[9]])
    gl, gr, gml, gmr, sr = _leads(b, Eg, p)
    temps = BP.initial_temperatures(L, 300.0, 310.0)
    h = 1e-3
    # The reference's Jacobian differentiates the occupations (and the
    # in-scattering escape rates) with G held fixed; with dsigma set to zero
    # it is the exact derivative of the fluxes at fixed probe self-energy.
    sw, dsw = BP.set_sigma_bp_w(temps, Eg, B_PROBE, 430.0)
    g = BP.g_full_probes(Eg, gl, gr, gml, gmr, sr, b["Hd"], b["Hdv"], b["Hld"], b["Hrd"], b["HR"], sw.T,
                         p["eta"], p["eta0"], 10.0)

    def fl_fixed(T):
        return BP.g_lesser(Eg, np.zeros(1, bool), gl, gr, g["GLeft"], g["G_full"], g["G_q_qp"], b["Hdv"],
                           b["Hld"], b["Hrd"], sw.T, np.zeros_like(dsw.T), T, 300.0, 310.0)["flux_i"][0]

    J0 = BP.g_lesser(Eg, np.zeros(1, bool), gl, gr, g["GLeft"], g["G_full"], g["G_q_qp"], b["Hdv"], b["Hld"],
                     b["Hrd"], sw.T, np.zeros_like(dsw.T), temps, 300.0, 310.0)["jacobian"][0]
    for j in range(L):
        tp, tm = temps.copy(), temps.copy()
        tp[j] += h
        tm[j] -= h
        fd = (fl_fixed(tp) - fl_fixed(tm)) / (2 * h)
        assert np.allclose(J0[:, j], fd, rtol=1e-5, atol=1e-9 * np.abs(J0).max())


def test_host_pieces_match_oracle():
    E = (np.arange(1, 34) / 33.0 * 20.0) ** 2
    x = np.sqrt(E)
    y = np.cos(x) + 1j * x
    assert abs(PB.simpson(x, y) - BP.simpson(x, y)) < 1e-12 * abs(BP.simpson(x, y))
    T = np.array([290.0, 305.0, 320.0])
    a, b_ = PB.sigma_probe(T, E, B_PROBE, 430.0)
    c, d = BP.set_sigma_bp_w(T, E, B_PROBE, 430.0)
    assert np.allclose(a, c, rtol=1e-14) and np.allclose(b_, d, rtol=1e-14)
    assert np.allclose(PB.initial_temperatures(5, 300, 310), BP.initial_temperatures(5, 300, 310))
    A = np.abs(np.random.default_rng(2).standard_normal((33, 3))) + 1.0
    Gn = A * np.stack([BP.bose_einstein(x, t) for t in (301.0, 299.0, 310.0)], axis=1)
    t1 = PB.lattice_temperatures(A, Gn, E, np.array([300.0, 300.0, 300.0]))
    t2 = BP.get_ph_temperature(A, Gn, E, np.array([300.0, 300.0, 300.0]))
    assert np.allclose(t1, t2, rtol=1e-10) and np.allclose(t1, [301.0, 299.0, 310.0], rtol=1e-6)
