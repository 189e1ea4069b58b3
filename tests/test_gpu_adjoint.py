"""GPU MP2 adjoint (dE/d(mu nu|lam sig), dE/dC) against the oracle, torch autograd and central
finite differences of the GPU energy itself."""
import numpy as np
import pytest

from oracle import adjoint as oadj
from juesgpu.synthetic import make_system, make_named

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mp():
    import juesgpu
    from juesgpu import MollerPlesset
    juesgpu.context(0)
    return MollerPlesset


def test_adjoint_matches_oracle(mp):
    s = make_system(16, 4, 48, seed=12)
    g, C, eps = np.array(s.ao_eri()), np.array(s.C), s.eps
    E, gb, cb = mp.rmp2_adjoint(gao=g, C=C, nocc=4, eps=eps, e_bar=0.75)
    Eo, gbo, cbo = oadj.mp2_adjoint(g, C, 4, eps, e_bar=0.75)
    assert abs(E - Eo) < 1e-14
    assert np.abs(gb - gbo).max() < 1e-13 * np.abs(gbo).max()
    assert np.abs(cb - cbo).max() < 1e-13 * np.abs(cbo).max()


def test_adjoint_matches_torch_autograd(mp):
    s = make_system(9, 3, 27, seed=13)
    g, C, eps = np.array(s.ao_eri()), np.array(s.C), s.eps
    E, gb, cb = mp.rmp2_adjoint(gao=g, C=C, nocc=3, eps=eps)
    Et, gbt, cbt = oadj.mp2_energy_torch(g, C, 3, eps)
    assert abs(E - Et) < 1e-14
    assert np.abs(gb - gbt).max() < 1e-13 * np.abs(gbt).max()
    assert np.abs(cb - cbt).max() < 1e-13 * np.abs(cbt).max()


def test_adjoint_split_precision(mp):
    # the split form (three planes in every transform and back-transform) against the FP64 oracle
    s = make_system(48, 10, 144, seed=14)
    g, C, eps = np.array(s.ao_eri()), np.array(s.C), s.eps
    E, gb, cb = mp.rmp2_adjoint(gao=g, C=C, nocc=10, eps=eps, precision="split")
    Eo, gbo, cbo = oadj.mp2_adjoint(g, C, 10, eps)
    assert abs(E - Eo) < 1e-7 * abs(Eo)
    assert np.linalg.norm(gb - gbo) < 3e-6 * np.linalg.norm(gbo)
    assert np.linalg.norm(cb - cbo) < 3e-6 * np.linalg.norm(cbo)


def energy(mp, g, C, o, eps):
    return mp.rmp2_adjoint(gao=g, C=C, nocc=o, eps=eps, want_gao=False, want_C=False)[0]


# bars of the central-difference checks (h = 1e-5, FP64 energies): the FP64 adjoint 1e-7
# relative; the split adjoint 1e-5 relative (its contractions keep ~2^-24 per GEMM)
FD_BAR = {"fp64": 1e-7, "split": 1e-5}


def test_adjoint_central_differences_nbf120(mp):
    # the adjoint in FP64 and in the split form, along 20 seeded unit directions, against central
    # differences of the FP64 GPU energy (the function both gradients approximate)
    s = make_named("ADJ120")
    o = s.nocc
    g, C, eps = np.asfortranarray(s.ao_eri()), np.array(s.C), s.eps
    grads = {p: mp.rmp2_adjoint(gao=g, C=C, nocc=o, eps=eps, precision=p)[1:] for p in FD_BAR}
    rng = np.random.default_rng(2024)
    h = 1e-5
    n = s.nbf
    worst = {p: 0.0 for p in FD_BAR}
    for k in range(20):
        if k % 2 == 0:
            # a symmetric ERI direction: d(B.B) for a random change of the factor B
            dB = rng.normal(size=s.B.shape)
            dB = dB + np.transpose(dB, (0, 2, 1))
            Bm = s.B.reshape(s.naux, n * n)
            dBm = dB.reshape(s.naux, n * n)
            d = (Bm.T @ dBm)
            d = (d + d.T).T.reshape(n, n, n, n, order="F")
            d /= np.linalg.norm(d)
            ep = energy(mp, g + h * d, C, o, eps)
            em = energy(mp, g - h * d, C, o, eps)
            which = 0
        else:
            d = rng.normal(size=C.shape)
            d /= np.linalg.norm(d)
            ep = energy(mp, g, C + h * d, o, eps)
            em = energy(mp, g, C - h * d, o, eps)
            which = 1
        fd = (ep - em) / (2 * h)
        for p, gr in grads.items():
            an = float(np.vdot(gr[which], d))
            rel = abs(fd - an) / max(abs(an), 1e-3 * np.linalg.norm(gr[which]))
            worst[p] = max(worst[p], rel)
    for p, bar in FD_BAR.items():
        assert worst[p] < bar, (p, worst)
