"""GPU CCSD from a general Fock matrix (AutoRCCSD.jl) and get_fock, against the oracle.

The oracle restates AutoRCCSD.jl's own auto-factorised update term by term; the GPU runs the
library's CCSD sweep with the non-canonical Fock terms added.  Both are the same CCSD map, so
they agree sweep by sweep.  Pins: the canonical H2O energy is the reference's CCSD known
answer, rotated orbitals give the same energy, frozen core matches the active-space CCSD.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import auto_rccsd
from juesgpu.Wavefunction import wfn_from_rhf
from juesgpu.synthetic import make_named

pytestmark = pytest.mark.gpu

E_CCSD_H2O = -0.070680102078571          # test/TestCoupledCluster.jl:44-45
E_PT_H2O_SPIN_ORBITAL = -9.987729603009741e-05


@pytest.fixture(scope="module")
def jg():
    import juesgpu
    from juesgpu import CoupledCluster, IntegralTransformation  # noqa: F401
    juesgpu.context(0)
    return juesgpu


def h2o_rotated(scale, seed=3):
    from scipy.linalg import expm
    d = np.load(os.path.join(GOLDEN, "h2o_sto3g.npz"))
    o, n = int(d["nocc"]), d["C"].shape[1]
    rng = np.random.default_rng(seed)
    Ao = rng.standard_normal((o, o))
    Av = rng.standard_normal((n - o, n - o))
    C = d["C"].copy()
    C[:, :o] = C[:, :o] @ expm(scale * (Ao - Ao.T))
    C[:, o:] = C[:, o:] @ expm(scale * (Av - Av.T))
    return wfn_from_rhf(C, d["eps"], d["ao_eri"], o, hao=d["H"])


@pytest.mark.parametrize("which", ["h2o", "h2o_rotated", "S25"])
def test_get_fock_matches_oracle(jg, which):
    if which == "S25":
        s = make_named("S25")
        w = s.wfn()
    else:
        w = h2o_rotated(0.0 if which == "h2o" else 0.1)
    f_gpu = jg.IntegralTransformation.get_fock(w)
    f_ref = auto_rccsd.get_fock(w.Ca, w.Cao, w.ao_eri, w.hao)
    assert np.abs(f_gpu - f_ref).max() < 1e-12 * max(1.0, np.abs(f_ref).max())


@pytest.mark.parametrize("scale,fcn", [(0.0, 0), (0.1, 0), (0.1, 1)])
def test_auto_rccsd_matches_oracle_sweep_by_sweep(jg, scale, fcn):
    from juesgpu.CoupledCluster import AutoRCCSD
    w = h2o_rotated(scale)
    ref_log = []
    e_ref, t1_ref, T2_ref, _, _ = auto_rccsd.do_rccsd(w, fcn=fcn, log=ref_log, return_T=True)
    e, t1, T2, log = AutoRCCSD.do_rccsd(w, fcn=fcn, return_T=True)
    assert len(log) == len(ref_log)
    for (it, en, rn, *_), (it_r, en_r, rn_r) in zip(log, ref_log):
        assert it == it_r
        assert abs(en - en_r) < 1e-11
        assert abs(rn - rn_r) < 1e-9 * max(rn_r, 1e-12) + 1e-16
    assert abs(e - e_ref) < 1e-11
    assert np.abs(t1 - t1_ref).max() < 1e-9 and np.abs(T2 - T2_ref).max() < 1e-9
    if fcn == 0:
        assert abs(e - E_CCSD_H2O) < 1e-9       # rotation invariance of the CCSD energy


def non_hf_synthetic(name, scale=0.01, seed=5):
    """A synthetic system whose core Hamiltonian makes the Fock matrix of its orbitals
    diag(eps) + delta (delta symmetric, |delta| ~ scale): a non-Hartree-Fock, non-canonical
    reference with a full occupied-virtual block.  (The generator's own H is unrelated to its
    orbitals.)"""
    s = make_named(name)
    g = s.ao_eri()
    C, o = s.C, s.nocc
    Co = C[:, :o]
    D = Co @ Co.T
    J = np.einsum("mnls,ls->mn", g, D, optimize=True)
    K = np.einsum("mlns,ls->mn", g, D, optimize=True)
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((s.nbf, s.nbf)) * scale
    f = np.diag(s.eps) + (d + d.T) / 2
    hao = C @ f @ C.T - 2.0 * J + K
    return wfn_from_rhf(C, s.eps, g, o, hao=hao), f


def test_auto_rccsd_pT_and_split(jg):
    from juesgpu.CoupledCluster import AutoRCCSD
    w = h2o_rotated(0.0)
    e, ept = AutoRCCSD.do_rccsd(w, do_pT=True)
    assert abs(e - E_CCSD_H2O) < 1e-9
    assert abs(ept - E_PT_H2O_SPIN_ORBITAL) < 1e-11
    # a non-HF reference at nbf=25: sweep by sweep against the oracle
    ws, f = non_hf_synthetic("S25")
    assert np.abs(jg.IntegralTransformation.get_fock(ws) - f).max() < 1e-10
    ref_log = []
    e_ref = auto_rccsd.do_rccsd(ws, cc_max_iter=12, log=ref_log)
    e, _, _, log = AutoRCCSD.do_rccsd(ws, cc_max_iter=12, return_T=True)
    for a, b in zip(log, ref_log):
        assert abs(a[1] - b[1]) < 1e-10 * max(1.0, abs(b[1]))
    # split precision at nbf=100 against the FP64 run
    w100, _ = non_hf_synthetic("S100")
    kw = dict(cc_max_iter=40, cc_e_conv=1e-9, cc_max_rms=1e-12, diis=True)
    e64 = AutoRCCSD.do_rccsd(w100, **kw)
    e_sp = AutoRCCSD.do_rccsd(w100, precision="split_bf16", **kw)
    assert abs(e_sp - e64) < 1e-6 * max(1.0, abs(e64))
