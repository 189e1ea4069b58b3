"""GPU parity of the FP64 (drop-in) form against the oracle and the reference's known answers.

Every call goes through the C ABI (juesgpu -> libjuesgpu.so).  Tolerances: 1e-10 Eh on
energies and 1e-9 on amplitudes (the drop-in bar); 1e-12 relative on integrals.
"""
import json
import os
import warnings

import numpy as np
import pytest

from conftest import GOLDEN
import oracle
from oracle import ccd as occd, ccsd as occsd
from oracle.mp2 import rmp2_energy
from juesgpu.Wavefunction import wfn_from_rhf
from juesgpu.synthetic import make_named, make_system

pytestmark = pytest.mark.gpu

E_MP2_H2O = -0.04914964480386458      # test/TestMollerPlesset.jl:35
E_CCD_H2O = -0.07015050066089029      # test/TestCoupledCluster.jl:41-42
E_CCSD_H2O = -0.070680102078571       # test/TestCoupledCluster.jl:44-45


@pytest.fixture(scope="module")
def jg():
    import juesgpu
    from juesgpu import CoupledCluster, IntegralTransformation, MollerPlesset, Transformation  # noqa
    juesgpu.context(0)
    return juesgpu


def h2o():
    d = np.load(os.path.join(GOLDEN, "h2o_sto3g.npz"))
    return wfn_from_rhf(d["C"], d["eps"], d["ao_eri"], int(d["nocc"]))


def golden():
    with open(os.path.join(GOLDEN, "synthetic_golden.json")) as f:
        return json.load(f)


# ------------------------------------------------------------------------------ transform
@pytest.mark.parametrize("n,dims", [(7, (2, 5, 3, 4)), (1, (1, 1, 1, 1)), (13, (13, 1, 6, 13)),
                                    (70, (9, 61, 9, 61))])
def test_tei_transform_matches_oracle(jg, n, dims):
    rng = np.random.default_rng(n)
    g = rng.normal(size=(n, n, n, n))          # no symmetry assumed
    Cs = [rng.normal(size=(n, d)) for d in dims]
    got = jg.Transformation.tei_transform(g, *Cs)
    want = oracle.tei_transform(g, *Cs)
    assert got.shape == want.shape
    assert np.allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())


def test_tei_transform_two_argument_form(jg):
    s = make_system(11, 3, 33, seed=2)
    g = s.ao_eri()
    a = jg.Transformation.tei_transform(g, s.C)
    b = jg.Transformation.tei_transform(g, s.C, s.C, s.C, s.C)
    assert np.array_equal(a, b)
    assert np.allclose(a, oracle.tei_transform(g, s.C), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("spec", ["OOVV", "VVVV", "OVVO", "OVOV", "OOOO", "ooov", "ovvv", "oovv"])
@pytest.mark.parametrize("notation", ["phys", "chem"])
def test_get_eri_blocks(jg, spec, notation):
    w = make_system(12, 3, 36, seed=5).wfn()
    got = jg.IntegralTransformation.get_eri(w, spec, notation)
    want = oracle.get_eri(w, spec, notation)
    assert got.shape == want.shape
    assert np.allclose(got, want, rtol=1e-12, atol=1e-14)


def test_get_eri_frozen_core(jg):
    w = make_system(12, 4, 36, seed=6).wfn()
    got = jg.IntegralTransformation.get_eri(w, "OOVV", fcn=2)
    assert np.allclose(got, oracle.get_eri(w, "OOVV", fcn=2), atol=1e-14)


def test_get_eri_rejects_bad_spec(jg):
    w = make_system(8, 2, 24).wfn()
    with pytest.raises(ValueError):
        jg.IntegralTransformation.get_eri(w, "OOVX")


# ------------------------------------------------------------------------------ MP2
def test_rmp2_h2o_known_answer(jg):
    assert abs(jg.MollerPlesset.do_rmp2(h2o()) - E_MP2_H2O) < 1e-10


@pytest.mark.parametrize("name", ["S25", "S100"])
def test_rmp2_synthetic(jg, name):
    w = make_named(name).wfn()
    want = golden()[name]["mp2"]
    assert abs(jg.MollerPlesset.do_rmp2(w) - want) < 1e-10 * max(1.0, abs(want))


def test_rmp2_odd_sizes(jg):
    for n, o in ((5, 1), (9, 4), (17, 8)):
        w = make_system(n, o, 3 * n, seed=n).wfn()
        assert abs(jg.MollerPlesset.do_rmp2(w) - oracle.do_rmp2(w)) < 1e-12


# ------------------------------------------------------------------------------ CCD
def test_rccd_h2o_known_answer(jg):
    from juesgpu.CoupledCluster import RCCD, mRCCD
    w = h2o()
    assert abs(mRCCD.do_rccd(w, maxit=100, r_conv=1e-12) - E_CCD_H2O) < 1e-10
    assert abs(RCCD.do_rccd(w) - E_CCD_H2O) < 1e-10          # 40 sweeps from (ij|ab)/D


# per-iteration energy bars: 1e-12 Eh at nbf=25 (|E| ~ 0.03), 1e-11 Eh at nbf=100 (|E| ~ 1.4,
# 10^6 more terms in each sum); step norms 1e-9 relative
EBAR = {"S25": 1e-12, "S100": 1e-11}


def check_log(log, ref, ebar):
    assert len(log) == len(ref)
    for (it, en, rn, ms, p), (rit, ren, rrn) in zip(log, ref):
        assert it == rit
        assert abs(en - ren) < ebar, (it, en, ren)
        assert abs(rn - rrn) < 1e-9 * max(1.0, rrn), (it, rn, rrn)


@pytest.mark.parametrize("name", ["S25", "S100"])
def test_rccd_per_iteration_matches_oracle(jg, name):
    # mRCCD.jl's driver: T2 = 0, DIIS (FP64) from the first sweep, 8 sweeps
    from juesgpu.CoupledCluster import mRCCD
    ref = golden()[name]["ccd_zero_diis_8"]
    w = make_named(name).wfn()
    e, log = mRCCD.do_rccd(w, maxit=8, r_conv=0.0, return_log=True)
    check_log(log, ref, EBAR[name])


@pytest.mark.parametrize("name", ["S25", "S100"])
def test_rccd_mp2_guess_diis_trajectory_matches_oracle(jg, name):
    # MP2 guess and DIIS to convergence: every sweep of the oracle's trajectory
    from juesgpu.CoupledCluster import mRCCD
    ref = golden()[name]["ccd_mp2guess_diis"]["log"]
    w = make_named(name).wfn()
    e, log = mRCCD.do_rccd(w, maxit=len(ref), r_conv=0.0, guess="mp2", return_log=True)
    check_log(log, ref, EBAR[name])


def test_rccd_amplitudes_match_oracle(jg):
    from juesgpu.CoupledCluster import mRCCD
    w = make_named("S25").wfn()
    e, T2 = mRCCD.do_rccd(w, maxit=60, r_conv=1e-11, return_T2=True, guess="mp2")
    eo, To, _ = occd.do_rccd(w, maxit=60, r_conv=1e-11, guess="mp2", return_T2=True)
    assert abs(e - eo) < 1e-10
    assert np.abs(T2 - To).max() < 1e-9
    # closed-shell pair symmetry T[i,j,a,b] = T[j,i,b,a]
    assert np.abs(T2 - np.transpose(T2, (1, 0, 3, 2))).max() < 1e-12


@pytest.mark.parametrize("name", ["S25", "S100"])
def test_rccd_converged_energy(jg, name):
    from juesgpu.CoupledCluster import mRCCD
    ref = golden()[name]["ccd_mp2guess_diis"]
    w = make_named(name).wfn()
    e = mRCCD.do_rccd(w, maxit=60, r_conv=1e-11, guess="mp2")
    assert abs(e - ref["energy"]) < 1e-10


def test_rccd_guesses_reach_same_energy(jg):
    from juesgpu.CoupledCluster import mRCCD
    w = make_named("S25").wfn()
    es = [mRCCD.do_rccd(w, maxit=80, r_conv=1e-11, guess=g) for g in ("zero", "mp2", "ovov")]
    assert max(es) - min(es) < 1e-11


# ------------------------------------------------------------------------------ CCSD
def test_rccsd_h2o_known_answer(jg):
    from juesgpu.CoupledCluster import RCCSD
    assert abs(RCCSD.do_rccsd(h2o()) - E_CCSD_H2O) < 1e-10


@pytest.mark.parametrize("name", ["S25", "S100"])
def test_rccsd_per_iteration_matches_oracle(jg, name):
    # RCCSD.jl's driver: T1 = 0, T2 = MP2, plain Jacobi sweeps
    from juesgpu.CoupledCluster._solve import solve
    ref = golden()[name]["ccsd_plain_6"]
    w = make_named(name).wfn()
    e, t1, T2, nit, log = solve(1, w, maxit=6, r_conv=0.0, diis=False, guess="mp2")
    check_log(log, ref, EBAR[name])


@pytest.mark.parametrize("name", ["S25", "S100"])
def test_rccsd_diis_trajectory_matches_oracle(jg, name):
    from juesgpu.CoupledCluster._solve import solve
    ref = golden()[name]["ccsd_diis"]["log"]
    w = make_named(name).wfn()
    e, t1, T2, nit, log = solve(1, w, maxit=len(ref), r_conv=0.0, diis=True, guess="mp2")
    check_log(log, ref, EBAR[name])


def test_rccsd_amplitudes_match_oracle(jg):
    from juesgpu.CoupledCluster import RCCSD
    w = make_named("S25").wfn()
    e, t1, T2 = RCCSD.do_rccsd(w, maxit=12, return_T1=True)
    eo, t1o, T2o, _ = occsd.do_rccsd(w, form="jl", maxit=12, return_T=True)
    assert abs(e - eo) < 1e-11
    assert np.abs(t1 - t1o).max() < 1e-10
    assert np.abs(T2 - T2o).max() < 1e-10


@pytest.mark.parametrize("name", ["S25", "S100"])
def test_rccsd_converged_energy(jg, name):
    from juesgpu.CoupledCluster import RCCSD
    ref = golden()[name]["ccsd_diis"]
    w = make_named(name).wfn()
    e = RCCSD.do_rccsd(w, maxit=60, diis=True, r_conv=1e-11)
    assert abs(e - ref["energy"]) < 1e-10


# ------------------------------------------------------------------------------ sessions
def test_session_single_sweeps_equal_whole_solve(jg):
    from juesgpu.CoupledCluster import CCSession, mRCCD
    w = make_named("S25").wfn()
    e_whole = mRCCD.do_rccd(w, maxit=6, r_conv=0.0, guess="mp2")
    s = CCSession(0, w, guess="mp2", r_conv=0.0, maxit=6)
    for _ in range(6):
        s.iterate(1)
    assert s.energy() == e_whole
    assert len(s.log()) == 6
    s.close()


# ------------------------------------------------------------------------------ errors
def test_dimension_errors(jg):
    from juesgpu import _lib
    import ctypes as C
    ctx = _lib.context(0)
    e = C.c_double()
    g = np.zeros((4, 4, 4, 4), order="F")
    c = np.zeros((4, 3), order="F")
    eps = np.zeros(4)
    st = ctx.lib.jues_rmp2(ctx.h, _lib.ptr(g), 4, _lib.ptr(c), 3, _lib.ptr(c), 3, _lib.ptr(eps), 0,
                           C.byref(e), None)
    assert st == _lib.EINVAL and "exceeds" in _lib.last_error()
    st = ctx.lib.jues_rmp2(ctx.h, None, 4, _lib.ptr(c), 1, _lib.ptr(c), 3, _lib.ptr(eps), 0,
                           C.byref(e), None)
    assert st == _lib.EINVAL and "null" in _lib.last_error()


def test_memory_cap_gives_enomem(jg):
    from juesgpu import _lib
    ctx = _lib.Context(0)
    ctx.set_mem_limit(1 << 20)
    w = make_named("S25").wfn()
    import ctypes as C
    g = _lib.f64(w.ao_eri)
    e = C.c_double()
    st = ctx.lib.jues_rmp2(ctx.h, _lib.ptr(g), 25, _lib.ptr(_lib.f64(w.Cao)), 5,
                           _lib.ptr(_lib.f64(w.Cav)), 20, _lib.ptr(_lib.f64(w.epsa)), 0, C.byref(e), None)
    assert st == _lib.ENOMEM
    ctx.set_mem_limit(0)
    st = ctx.lib.jues_rmp2(ctx.h, _lib.ptr(g), 25, _lib.ptr(_lib.f64(w.Cao)), 5,
                           _lib.ptr(_lib.f64(w.Cav)), 20, _lib.ptr(_lib.f64(w.epsa)), 0, C.byref(e), None)
    assert st == _lib.OK
    ctx.close()


def test_non_convergence_is_reported(jg):
    from juesgpu.CoupledCluster import mRCCD
    w = make_named("S25").wfn()
    with warnings.catch_warnings(record=True) as rec:
        warnings.simplefilter("always")
        e = mRCCD.do_rccd(w, maxit=1, r_conv=1e-12)
    assert any("converge" in str(r.message) for r in rec)
    assert np.isfinite(e)


def test_nonfinite_input_is_rejected(jg):
    from juesgpu import JuESError
    from juesgpu.CoupledCluster import mRCCD
    w = make_system(8, 2, 24).wfn()
    w.ao_eri[0, 0, 0, 0] = np.nan
    with pytest.raises(JuESError) as ei:
        mRCCD.do_rccd(w, maxit=3)
    assert ei.value.code == 5


# ------------------------------------------------------------------------------ DF-MP2
def _df_inputs(s, rotate):
    """pqP, Jpqh for a synthetic system: its integrals are exactly sum_P B_P (x) B_P, so
    DF-MP2 with the fitted b = B is exact.  ``rotate`` hides b behind an orthogonal Jpqh:
    pqP = b Q^T and Jpqh = Q give pqP Jpqh = b."""
    b = np.transpose(s.B, (1, 2, 0))
    if not rotate:
        return np.asfortranarray(b), None
    rng = np.random.default_rng(7)
    Q, _ = np.linalg.qr(rng.standard_normal((s.naux, s.naux)))
    return np.asfortranarray(np.einsum("pqQ,PQ->pqP", b, Q)), np.asfortranarray(Q)


@pytest.mark.parametrize("name,rotate", [("S25", False), ("S25", True), ("S100", True)])
def test_df_rmp2_equals_conventional_on_exact_factorisation(jg, name, rotate):
    # TestMollerPlesset.jl:38-39 checks the DF form against the same molecule's MP2
    s = make_named(name)
    pqP, Jpqh = _df_inputs(s, rotate)
    w = s.wfn()
    e_df = jg.MollerPlesset.do_df_rmp2(w, pqP, Jpqh)
    ref = golden()[name]["mp2"]
    assert abs(e_df - ref) < 1e-10 * max(1.0, abs(ref))
    if name == "S25":
        assert abs(e_df - oracle.df_rmp2(w, pqP, Jpqh)) < 1e-12
    e_split = jg.MollerPlesset.do_df_rmp2(w, pqP, Jpqh, precision="split_bf16")
    assert abs(e_split - ref) < 1e-6


def test_df_rmp2_rejects_bad_shapes(jg):
    s = make_named("S25")
    w = s.wfn()
    with pytest.raises(ValueError):
        jg.MollerPlesset.do_df_rmp2(w, np.zeros((25, 24, 75)))
    with pytest.raises(ValueError):
        jg.MollerPlesset.do_df_rmp2(w, np.zeros((25, 25, 75)), np.zeros((75, 74)))


# ------------------------------------------------------------------------------ DF-CCD
def test_df_rccd_matches_oracle_sweep_by_sweep(jg):
    # DF-RCCD.jl as written (its WmBeJ), through an orthogonal Jpqh
    from oracle import df_rccd
    from juesgpu.CoupledCluster import solve_df
    s = make_named("S25")
    pqP, Jpqh = _df_inputs(s, True)
    w = s.wfn()
    e, T2, nit, log = solve_df(w, pqP, Jpqh, maxit=8, guess="mp2", diis=False, r_conv=0.0)
    ref_log = []
    e_ref, T_ref = df_rccd.do_df_rccd(w, np.einsum("pqP,PQ->pqQ", pqP, Jpqh), maxit=8, return_T2=True,
                                      log=ref_log)
    assert nit == 8
    for (it, en, *_), (it_r, en_r) in zip(log, ref_log):
        assert it == it_r and abs(en - en_r) < 1e-10 * max(1.0, abs(en_r))
    assert abs(e - e_ref) < 1e-10
    assert np.abs(T2 - T_ref).max() < 1e-9
    # the mirror's defaults are the reference's: 40 sweeps, MP2 guess, no DIIS
    e40 = jg.CoupledCluster.DFRCCD.do_df_rccd(w, pqP, Jpqh)
    assert abs(e40 - df_rccd.do_df_rccd(w, np.transpose(s.B, (1, 2, 0)), maxit=40)) < 1e-10


@pytest.mark.parametrize("name", ["S25", "S100"])
def test_df_rccd_rccd_variant_equals_conventional(jg, name):
    # with RCCD.jl's WmBeJ, CCD on exactly factorised integrals is conventional CCD
    from juesgpu.CoupledCluster import solve, solve_df
    s = make_named(name)
    pqP, _ = _df_inputs(s, False)
    w = s.wfn()
    kw = dict(maxit=6, guess="mp2", diis=False, r_conv=0.0)
    _, T_df, _, log_df = solve_df(w, pqP, None, variant="rccd", **kw)
    _, _, T_ao, _, log_ao = solve(0, w, **kw)
    for a, b in zip(log_df, log_ao):
        assert abs(a[1] - b[1]) < 1e-10 * max(1.0, abs(b[1]))
    assert np.abs(T_df - T_ao).max() < 1e-9


def test_df_rccd_split_precision(jg):
    from juesgpu.CoupledCluster import solve_df
    s = make_named("S100")
    pqP, Jpqh = _df_inputs(s, True)
    w = s.wfn()
    kw = dict(maxit=40, guess="mp2", diis=True, r_conv=1e-9)
    e64 = solve_df(w, pqP, Jpqh, **kw)[0]
    e_split = solve_df(w, pqP, Jpqh, precision="split_bf16", transform_precision="fp64", refine=2, **kw)[0]
    assert abs(e_split - e64) < 1e-6


def test_df_rccd_session_and_errors(jg):
    from juesgpu.CoupledCluster import CCSession
    s = make_named("S25")
    pqP, _ = _df_inputs(s, False)
    w = s.wfn()
    ses = CCSession(0, w, pqP=pqP, guess="mp2", diis=False, r_conv=0.0, maxit=3)
    ses.iterate(3)
    e3 = ses.energy()
    ses.close()
    assert abs(e3 - jg.CoupledCluster.DFRCCD.do_df_rccd(w, pqP, maxit=3)) < 1e-12
    with pytest.raises(ValueError):
        CCSession(1, w, pqP=pqP)
    with pytest.raises(KeyError):
        jg.CoupledCluster.DFRCCD.do_df_rccd(w, pqP, variant="nope")


# ------------------------------------------------------------------------------ Wfn{Float32}
def f32_wfn(w):
    """The Wfn{Float32} the reference's tests build (test/TestCoupledCluster.jl:23): every array
    rounded to single precision."""
    return wfn_from_rhf(w.Ca, w.epsa, w.ao_eri, w.nalpha, dtype=np.float32)


def test_float32_wfn_through_the_c_abi(jg):
    # Float32 arrays are promoted to FP64 on the way in (exactly), so the GPU must match the oracle
    # run on the same rounded inputs at the drop-in bar
    from juesgpu import MollerPlesset
    from juesgpu.CoupledCluster import RCCSD, mRCCD
    w32 = f32_wfn(make_named("S25").wfn())
    assert w32.ao_eri.dtype == np.float32 and w32.Cao.dtype == np.float32
    w64 = wfn_from_rhf(w32.Ca.astype(np.float64), w32.epsa.astype(np.float64),
                       w32.ao_eri.astype(np.float64), w32.nalpha)
    assert abs(MollerPlesset.do_rmp2(w32) - oracle.do_rmp2(w64)) < 1e-12
    e_ccd = mRCCD.do_rccd(w32, maxit=60, r_conv=1e-11, guess="mp2")
    assert abs(e_ccd - occd.do_rccd(w64, maxit=60, r_conv=1e-11, guess="mp2")) < 1e-10
    e_ccsd = RCCSD.do_rccsd(w32, maxit=60, diis=True, r_conv=1e-11)
    assert abs(e_ccsd - occsd.do_rccsd(w64, form="jl", maxit=60, diis=True, r_conv=1e-11)) < 1e-10


def test_float32_h2o_close_to_the_known_answers(jg):
    # the rounding of the inputs moves the H2O energies by far less than the reference's own
    # FP32-vs-FP64 gap (7.8e-9 Eh for RCCD, test/TestCoupledCluster.jl:41-46)
    from juesgpu import MollerPlesset
    from juesgpu.CoupledCluster import mRCCD
    w32 = f32_wfn(h2o())
    assert abs(MollerPlesset.do_rmp2(w32) - E_MP2_H2O) < 1e-6
    assert abs(mRCCD.do_rccd(w32, maxit=100, r_conv=1e-12) - E_CCD_H2O) < 1e-6


# ------------------------------------------------------------------------------ mRCCSD.jl's Fae
def test_mrccsd_fae_variant_matches_oracle(jg):
    # mRCCSD.jl:140 contracts t1 with <me|af> in Fae where RCCSD.jl:190 uses <ma|ef>; the mirror of
    # mRCCSD runs the former, checked sweep by sweep and converged against the oracle's mRCCSD form
    from juesgpu.CoupledCluster import mRCCSD, RCCSD
    from juesgpu.CoupledCluster._solve import solve
    for name in ("S25", "S100"):
        g = golden()[name]
        w = make_named(name).wfn()
        e, t1, T2, nit, log = solve(1, w, maxit=6, r_conv=0.0, diis=False, guess="mp2", ccsd_fae="mrccsd")
        check_log(log, g["ccsd_m_plain_6"], EBAR[name])
        e_m = mRCCSD.do_rccsd(w, maxit=60, diis=True, r_conv=1e-11)
        assert abs(e_m - g["ccsd_m_diis"]["energy"]) < 1e-10
        e_r = RCCSD.do_rccsd(w, maxit=60, diis=True, r_conv=1e-11)
        assert abs(e_r - g["ccsd_diis"]["energy"]) < 1e-10
