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
    assert info1.tuned == 1 and info1.nstages == 4 and info1.graph_nodes == 5
    for (g, C, o, eps), e in zip(sy, e1):
        assert abs(e - oadj.mp2_energy(g, C, o, eps)) < 1e-13
    e2, _, _, info2 = mp.batch_rmp2(sy)
    assert info2.tuned == 0
    assert np.array_equal(e1, e2)


def test_batch_adjoint_matches_single_system(mp):
    sy = systems(16, 6, 18, seed=9)
    e, gbs, cbs, info = mp.batch_rmp2(sy, adjoint=True, e_bar=0.5)
    assert info.nstages == 12 and info.graph_nodes == 13
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
