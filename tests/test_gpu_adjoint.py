"""GPU adjoint of the transmission and of the Landauer conductance: against
the oracle's adjoint (FP64) and against central finite differences."""
import numpy as np
import pytest

from oracle import adjoint as A
from phinfortran_gb300 import systems as S
from phinfortran_gb300 import transport_tdb
from phinfortran_gb300.gradients import conductance_fn, landauer_weights, transport_grad

pytestmark = pytest.mark.gpu


def small_bar(seed=4):
    return S.sc_phonon(nx=2, ny=2, L=5, ne=16, mass_range=(1, 3), bond_range=(0.8, 1.2), seed_index=seed)


@pytest.mark.parametrize("ckpt,arith", [(1, "fp64"), (0, "fp64"), (3, "fp64"), (7, "fp64"), (1, "df64"),
                                        (0, "df64"), (2, "df64")])
def test_sensitivities_match_oracle(cuda_ready, ckpt, arith):
    """ckpt = 1 keeps every layer; 0 checkpoints every ceil(sqrt(L+2)) = 3
    layers and recomputes; 3 with L = 5 leaves a short last segment; 7 is
    one segment (kept from the forward pass, nothing recomputed); 2 four
    segments.  df64: every block operation in double-float (about 48 bits)."""
    b, E, p, aux = small_bar()
    Es = E[2:14]
    w = np.linspace(0.3, 1.7, Es.size)
    T, M, st = transport_grad(Es, b, w, ckpt=ckpt, arith=arith, **p)
    To, Mo = A.transport_and_sensitivities(Es, b, p["eta"], p["eta0"], p["convergence"], p["dev_factor"])
    assert (st == 0).all()
    tol_t, tol_m = (1e-10, 1e-9) if arith == "fp64" else (1e-9, 1e-7)
    np.testing.assert_allclose(T, To, rtol=tol_t, atol=1e-12)
    for k in ("Hd", "Hdv", "Hld", "Hrd"):
        ref = np.tensordot(w, Mo[k], axes=(0, 0))
        got = M[k][0]
        scale = np.abs(ref).max()
        assert np.abs(got - ref).max() <= tol_m * scale, (k, np.abs(got - ref).max(), scale)


@pytest.mark.parametrize("arith", ["fp64", "df64"])
def test_conductance_gradient_vs_finite_differences(cuda_ready, arith):
    import torch
    b, E, p, aux = small_bar(seed=6)
    bar, m0, k0 = aux["bar"], aux["masses"], aux["springs"]
    omega = aux["omega"][1:]
    temp = 300.0
    fn = conductance_fn()
    m = torch.tensor(m0, requires_grad=True)
    k = torch.tensor(k0, requires_grad=True)
    kappa = fn.apply(m, k, bar, omega, temp, p, "fp64", arith)
    kappa.backward()
    gm, gk = m.grad.numpy(), k.grad.numpy()
    wts = landauer_weights(omega, temp)

    def kap(mm, kk):
        r = transport_tdb(omega ** 2, bar.blocks(mm, kk), want_transr=False, **p)
        return float(np.dot(wts, r["transl"]))

    h = 1e-6
    for i in bar.dev_atoms[[0, 7, 13, 19]]:
        mp, mn = m0.copy(), m0.copy()
        mp[i] += h
        mn[i] -= h
        fd = (kap(mp, k0) - kap(mn, k0)) / (2 * h)
        assert abs(fd - gm[i]) <= 1e-5 * max(abs(fd), abs(gm).max()), (i, fd, gm[i])
    for j in np.nonzero(bar.dev_bond & (bar.bonds[:, 2] == 2))[0][:4]:
        kp, kn = k0.copy(), k0.copy()
        kp[j] += h
        kn[j] -= h
        fd = (kap(m0, kp) - kap(m0, kn)) / (2 * h)
        assert abs(fd - gk[j]) <= 1e-5 * max(abs(fd), abs(gk).max()), (j, fd, gk[j])
    # lead atoms and lead bonds carry no gradient (the leads are held fixed)
    lead_atoms = np.setdiff1d(np.arange(m0.size), bar.dev_atoms)
    assert np.all(gm[lead_atoms][:bar.nc * 2] == 0)
