"""Batched MP2 (one CUDA graph of grouped persistent launches) against the single-system path
and the oracle; a repeated batch replays the cached graph with identical results."""
import numpy as np
import pytest

from oracle import adjoint as oadj
from juesgpu.synthetic import batch_specs, make_system

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mp():
    import juesgpu
    from juesgpu import MollerPlesset
    juesgpu.context(0)
    return MollerPlesset


def systems(count, nmin, nmax, seed=5):
    out = []
    for n, o, naux, sub in batch_specs(count, seed=seed, nmin=nmin, nmax=nmax):
        s = make_system(n, o, naux, seed=sub)
        out.append((np.asfortranarray(s.ao_eri()), np.asfortranarray(s.C), o, s.eps))
    return out


def test_batch_energies_match_oracle_and_replay(mp):
    sy = systems(24, 6, 22)
    e1, _, _, info1 = mp.batch_rmp2(sy)
    # 4 grouped GETT stages + the Gamma/energy kernel and the per-system energy sum
    assert info1.tuned == 1 and info1.nstages == 4 and info1.graph_nodes == 6
    for (g, C, o, eps), e in zip(sy, e1):
        assert abs(e - oadj.mp2_energy(g, C, o, eps)) < 1e-13
    e2, _, _, info2 = mp.batch_rmp2(sy)
    assert info2.tuned == 0
    assert np.array_equal(e1, e2)


def test_batch_adjoint_matches_single_system(mp):
    sy = systems(16, 6, 18, seed=9)
    e, gbs, cbs, info = mp.batch_rmp2(sy, adjoint=True, e_bar=0.5)
    assert info.nstages == 12 and info.graph_nodes == 14
    for (g, C, o, eps), eb, gb, cb in zip(sy, e, gbs, cbs):
        E, gs, cs = mp.rmp2_adjoint(gao=g, C=C, nocc=o, eps=eps, e_bar=0.5)
        assert abs(E - eb) < 1e-13
        assert np.abs(gb - gs).max() < 1e-13 * np.abs(gs).max()
        assert np.abs(cb - cs).max() < 1e-13 * np.abs(cs).max()


def test_batch_rejects_bad_system(mp):
    from juesgpu import JuESError
    g = np.zeros((4, 4, 4, 4), order="F")
    C = np.eye(4, order="F")
    with pytest.raises(JuESError):
        mp.batch_rmp2([(g, C, 4, np.zeros(4))])


@pytest.mark.parametrize("form", ["tcgen05", "auto"])
def test_batch_split_grouped_tcgen05_matches_fp64(mp, form):
    # split precision: the grouped three-plane tcgen05 GEMM (pinned, or as the autotuner picks)
    # against the single-system FP64 adjoint; energies within 1e-9 Eh, gradients 1e-7 relative
    from juesgpu import _lib
    sy = systems(20, 10, 40, seed=3)
    ctx = _lib.context(0)
    ctx.set_batch_form(form)
    try:
        e, gbs, cbs, info = mp.batch_rmp2(sy, adjoint=True, e_bar=0.5, precision="split")
        e2, gbs2, cbs2, info2 = mp.batch_rmp2(sy, adjoint=True, e_bar=0.5, precision="split")
    finally:
        ctx.set_batch_form("auto")
    shapes = [info.tile_shape[k] for k in range(info.nstages)]
    if form == "tcgen05":
        # every stage but the final dE/dC one has K <= nbf <= 64
        assert shapes[:-1] == [4] * (info.nstages - 1), shapes
    assert info2.tuned == 0 and np.array_equal(e, e2)
    for (g, C, o, eps), eb, gb, cb in zip(sy, e, gbs, cbs):
        E, gs, cs = mp.rmp2_adjoint(gao=g, C=C, nocc=o, eps=eps, e_bar=0.5)
        assert abs(E - eb) < 1e-9, (E, eb)
        assert np.linalg.norm(gb - gs) < 1e-7 * np.linalg.norm(gs)
        assert np.linalg.norm(cb - cs) < 1e-7 * np.linalg.norm(cs)
