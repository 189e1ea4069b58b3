"""GPU (T) energy correction (compute_pT, PerturbativeTriples.jl:35-138) against the oracle.

The oracle's closed-shell (T) is pinned to an independent spin-orbital (T) on H2O/STO-3G
(tests/test_oracle.py); here the C-ABI path is checked against it: host-array entry point and
CCSD sessions, FP64 (1e-12 relative) and split precision (1e-6 relative).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import ccsd, triples
from juesgpu.Wavefunction import wfn_from_rhf
from juesgpu.synthetic import make_named

pytestmark = pytest.mark.gpu

E_PT_H2O_SPIN_ORBITAL = -9.987729603009741e-05   # independent spin-orbital (T), tests/test_oracle.py


@pytest.fixture(scope="module")
def jg():
    import juesgpu
    from juesgpu import CoupledCluster  # noqa: F401
    juesgpu.context(0)
    return juesgpu


def h2o():
    d = np.load(os.path.join(GOLDEN, "h2o_sto3g.npz"))
    return wfn_from_rhf(d["C"], d["eps"], d["ao_eri"], int(d["nocc"]))


def _inputs(w, t1, T2):
    oooo, ooov, oovv, ovov, ovvv, vvvv = ccsd.make_rccsd_integrals(w)
    Vvvvo, Vvooo, Vvovo = triples.integrals_from_cc(ovvv, ooov, oovv)
    o = w.nalpha
    return dict(T1=t1, T2=T2, Vvvvo=Vvvvo, Vvooo=Vvooo, Vvovo=Vvovo, fo=w.epsa[:o], fv=w.epsa[o:])


def test_pT_h2o_host_arrays_and_session(jg):
    from juesgpu.CoupledCluster import CCSession, PerturbativeTriples
    w = h2o()
    e, t1, T2, _ = ccsd.do_rccsd(w, return_T=True)
    kw = _inputs(w, t1, T2)
    e_ref = triples.compute_pT(**kw)
    assert abs(e_ref - E_PT_H2O_SPIN_ORBITAL) < 1e-13
    e_gpu = PerturbativeTriples.compute_pT(**kw)
    assert abs(e_gpu - e_ref) < 1e-14
    # a CCSD session converged on the GPU gives the same (T) from its resident blocks
    ses = CCSession(1, w, maxit=60, diis=True, r_conv=1e-11)
    ses.iterate(60)
    assert abs(ses.pT() - e_ref) < 1e-11
    ses.close()


def test_pT_synthetic_matches_oracle(jg):
    from juesgpu.CoupledCluster import PerturbativeTriples
    w = make_named("S25").wfn()
    e, t1, T2, _ = ccsd.do_rccsd(w, maxit=12, return_T=True)
    kw = _inputs(w, t1, T2)
    e_ref = triples.compute_pT(**kw)
    e_gpu = PerturbativeTriples.compute_pT(**kw)
    assert abs(e_gpu - e_ref) < 1e-12 * abs(e_ref)
    e_split = PerturbativeTriples.compute_pT(precision="split_bf16", **kw)
    assert abs(e_split - e_ref) < 1e-6 * abs(e_ref)


def test_pT_split_precision_s100_session(jg):
    from juesgpu.CoupledCluster import CCSession
    w = make_named("S100").wfn()
    ses = CCSession(1, w, maxit=8, diis=True, r_conv=0.0)
    ses.iterate(8)
    e64 = ses.pT("fp64")
    e_split = ses.pT("split_bf16")
    ses.close()
    assert e64 < 0
    assert abs(e_split - e64) < 1e-6 * abs(e64)


def test_pT_rejects_bad_shapes_and_ccd_sessions(jg):
    from juesgpu.CoupledCluster import CCSession, PerturbativeTriples
    w = h2o()
    e, t1, T2, _ = ccsd.do_rccsd(w, return_T=True)
    kw = _inputs(w, t1, T2)
    kw["Vvooo"] = kw["Vvooo"][:, :, :, :-1]
    with pytest.raises(ValueError):
        PerturbativeTriples.compute_pT(**kw)
    ses = CCSession(0, w, maxit=2)
    with pytest.raises(Exception):
        ses.pT()
    ses.close()
