"""Tight-binding oracle (oracle/tb.py, restating tb/hamiltonian.f90): the
Slater-Koster table is checked for rotational invariance (the spectrum of a
two-atom cluster with s, p, d, s* orbitals does not depend on the bond
direction) and gen_ham's Bloch sum for Hermiticity and a square-lattice
s band."""
import numpy as np

from oracle import tb as TB


def params(ns=1, seed=0):
    rng = np.random.default_rng(seed)
    V = rng.uniform(-2, 2, size=(ns, ns, 4, 4, 4))
    V = 0.5 * (V + np.swapaxes(V, 0, 1))
    V = 0.5 * (V + np.swapaxes(V, 2, 3))          # V(n1, n2) = V(n2, n1): a symmetric parameter set
    Vn = rng.uniform(1.0, 3.0, size=(ns, ns, 4, 4, 4))
    Vn = 0.5 * (Vn + np.swapaxes(Vn, 0, 1))
    Vn = 0.5 * (Vn + np.swapaxes(Vn, 2, 3))
    r_d = np.full((ns, ns), 2.35e-10)   # metres, positions in Angstrom (as the reference holds them)
    return V, Vn, r_d


def cluster_h(V, Vn, r_d, r):
    orbs = list(range(10))
    n = len(orbs)
    H = np.zeros((2 * n, 2 * n))
    for a, oa in enumerate(orbs):
        for b, ob in enumerate(orbs):
            H[a, b] = TB.onsite(V, 0, 0, oa, ob)
            H[n + a, n + b] = TB.onsite(V, 0, 0, oa, ob)
            H[a, n + b] = TB.v_sk(V, Vn, r_d, 0, 0, oa, ob, r)
            H[n + a, b] = TB.v_sk(V, Vn, r_d, 0, 0, oa, ob, -r)
    return 0.5 * (H + H.T)


def test_slater_koster_rotational_invariance():
    V, Vn, r_d = params()
    rng = np.random.default_rng(5)
    ref = None
    for _ in range(6):
        u = rng.normal(size=3)
        r = 2.4 * u / np.linalg.norm(u)
        ev = np.linalg.eigvalsh(cluster_h(V, Vn, r_d, r))
        if ref is None:
            ref = ev
        # float32 sqrt(3) in the table limits the invariance to ~1e-7 relative
        assert np.abs(ev - ref).max() < 1e-6 * np.abs(ref).max(), np.abs(ev - ref).max()


def test_gen_ham_square_lattice_s_band():
    """2 x 2 supercell of a square lattice (a = 2.5 A), one s orbital,
    nearest-neighbour V_ss_sigma = t, no distance scaling: the Hermitised
    H(k) has the folded band eps + 2t(cos kx a + cos ky a)."""
    a = 2.5
    V = np.zeros((1, 1, 4, 4, 4))
    V[0, 0, 0, 0, 0] = 0.3        # onsite s
    V[0, 0, 0, 0, 1] = -1.0       # ss sigma
    Vn = np.zeros_like(V)
    r_d = np.ones((1, 1))
    lat = np.array([[2 * a, 0, 0], [0, 2 * a, 0], [0, 0, 40 * a]])
    pos = np.array([[0, 0, 0], [a, 0, 0], [0, a, 0], [a, a, 0]], dtype=float)
    rec = 2 * np.pi * np.linalg.inv(lat).T
    for kf in ([0.0, 0.0, 0.0], [0.13, -0.31, 0.0], [0.5, 0.25, 0.0]):
        H = TB.gen_ham(pos, [0, 0, 0, 0], [[0]], V, Vn, r_d, lat, 1.1 * a, np.array(kf), rec)
        assert np.abs(H - H.conj().T).max() < 1e-15
        kc = np.array(kf) @ rec
        ev = np.sort(np.linalg.eigvalsh(H))
        want = np.sort([0.3 - 2 * (np.cos((kc[0] + gx) * a) + np.cos((kc[1] + gy) * a))
                        for gx in (0, np.pi / a) for gy in (0, np.pi / a)])
        np.testing.assert_allclose(ev, want, atol=1e-12)
