"""CPU tests of the oracle: pinned to the reference's known answers and cross-checked
between the reference's independent forms (no GPU)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
import oracle
from oracle import ccd, ccsd
from oracle.mp2 import rmp2_energy, rmp2_energy_loops
from juesgpu.Wavefunction import wfn_from_rhf
from juesgpu.synthetic import make_system, make_named


def h2o():
    d = np.load(os.path.join(GOLDEN, "h2o_sto3g.npz"))
    return wfn_from_rhf(d["C"], d["eps"], d["ao_eri"], int(d["nocc"]))


# reference known answers (psi4 integrals, see tests/golden/make_sto3g_fixtures.py)
E_MP2_H2O = -0.04914964480386458      # test/TestMollerPlesset.jl:35
E_CCD_H2O = -0.07015050066089029      # test/TestCoupledCluster.jl:41-42
E_CCSD_H2O = -0.070680102078571       # test/TestCoupledCluster.jl:44-45


def test_h2_ao_integrals_pin():
    g = np.load(os.path.join(GOLDEN, "h2_sto3g.npz"))["ao_eri"]
    # test/TestWavefunction.jl:33-35 (1-based Julia indices)
    assert abs(g[0, 0, 0, 0] - 0.7746059439198979) < 1e-12
    assert abs(g[1, 0, 1, 1] - 0.3093089669634818) < 1e-12
    assert abs(g[0, 0, 1, 1] - 0.4780413730018048) < 1e-12


def test_h2o_rmp2_pin():
    assert abs(oracle.do_rmp2(h2o()) - E_MP2_H2O) < 1e-10


def test_h2o_rccd_pin_both_forms():
    w = h2o()
    e_m = ccd.do_rccd(w, maxit=100, r_conv=1e-12)
    e_jl = ccd.do_rccd_jl(w)
    assert abs(e_m - E_CCD_H2O) < 1e-10
    assert abs(e_jl - E_CCD_H2O) < 1e-10


def test_h2o_rccsd_pin_both_forms():
    w = h2o()
    assert abs(ccsd.do_rccsd(w, form="m") - E_CCSD_H2O) < 1e-10
    assert abs(ccsd.do_rccsd(w, form="jl") - E_CCSD_H2O) < 1e-10


def test_tei_transform_two_arg_equals_four_arg():
    # TestTransformation.jl:31-62 analogue: RHF-via-1C == RHF-via-4C
    s = make_system(8, 2, 24, seed=3)
    g = s.ao_eri()
    a = oracle.tei_transform(g, s.C)
    b = oracle.tei_transform(g, s.C, s.C, s.C, s.C)
    assert np.array_equal(a, b)


def test_tei_transform_quarter_order_matches_direct_einsum():
    s = make_system(7, 2, 21, seed=4)
    g = s.ao_eri()
    rng = np.random.default_rng(0)
    Cs = [rng.normal(size=(7, d)) for d in (2, 5, 3, 4)]
    ref = np.einsum("mnls,mi,na,lj,sb->iajb", g, *Cs)
    assert np.allclose(oracle.tei_transform(g, *Cs), ref, rtol=1e-13, atol=1e-14)


def test_get_eri_blocks_are_slices_of_full_transform():
    s = make_system(9, 3, 27, seed=5)
    w = s.wfn()
    full = oracle.tei_transform(w.ao_eri, s.C)          # chem over all MOs
    phys = np.transpose(full, (0, 2, 1, 3))             # <pq|rs>
    o = 3
    sl = {"o": slice(0, o), "O": slice(0, o), "v": slice(o, 9), "V": slice(o, 9)}
    for spec in ("OOVV", "VVVV", "OVVO", "OVOV", "OOOO", "ooov", "ovvv", "vvvv"):
        blk = oracle.get_eri(w, spec)
        want = phys[tuple(sl[c] for c in spec)]
        assert np.allclose(blk, want, atol=1e-14), spec
        chem = oracle.get_eri(w, spec, notation="chem")
        assert np.allclose(chem, full[tuple(sl[c] for c in spec)], atol=1e-14), spec


def test_get_eri_frozen_core_and_bad_spec():
    s = make_system(9, 3, 27, seed=6)
    w = s.wfn()
    a = oracle.get_eri(w, "OOVV", fcn=1)
    b = oracle.get_eri(w, "OOVV")
    assert a.shape == (2, 2, 6, 6)
    assert np.allclose(a, b[1:, 1:], atol=1e-14)
    with pytest.raises(ValueError):
        oracle.get_eri(w, "OOV")
    with pytest.raises(ValueError):
        oracle.get_eri(w, "OOVX")


def test_rmp2_loop_equals_vectorised():
    s = make_system(8, 3, 24, seed=7)
    w = s.wfn()
    K = oracle.get_eri(w, "OOVV")
    assert abs(rmp2_energy(K, w.epsa, 3) - rmp2_energy_loops(K, w.epsa, 3)) < 1e-14


def test_ccd_forms_agree_per_iteration():
    s = make_named("S25")
    w = s.wfn()
    ints = ccd.make_rccd_integrals(w)
    ints_jl = ccd.make_rccd_integrals_jl(w.ao_eri, w.Cao, w.Cav)
    for a, b in zip(ints, ints_jl):
        assert np.allclose(a, b, atol=1e-14)
    la, lb = [], []
    ccd.do_rccd(w, maxit=6, r_conv=None, log=la, integrals=ints, form="m")
    ccd.do_rccd(w, maxit=6, r_conv=None, log=lb, integrals=ints, form="jl")
    for (_, ea, ra), (_, eb, rb) in zip(la, lb):
        assert abs(ea - eb) < 1e-13 and abs(ra - rb) < 1e-12


def test_ccd_zero_guess_first_iterate_is_mp2():
    # mRCCD.jl:245: T2 = 0, so the first sweep yields the MP2 amplitudes
    s = make_system(10, 3, 30, seed=8)
    w = s.wfn()
    ints = ccd.make_rccd_integrals(w)
    D = oracle.mp2.denominators(w.epsa, 3)
    T1 = ccd.m_residual_update(np.zeros_like(ints[0]), *ints[:1], ints[4], ints[3], ints[1],
                               ints[2], D)
    assert np.allclose(T1, ints[0] / D, atol=1e-15)
    assert abs(ccd.ccenergy(T1, ints[0]) - oracle.do_rmp2(w)) < 1e-13


def test_ccd_guesses_converge_to_same_point():
    w = make_named("S25").wfn()
    ints = ccd.make_rccd_integrals(w)
    es = [ccd.do_rccd(w, maxit=80, r_conv=1e-11, guess=g, integrals=ints)
          for g in ("zero", "mp2", "ovov")]
    assert max(es) - min(es) < 1e-11


def test_ccd_fp32_diis_as_reference_is_close():
    # the reference's Float32 DIIS (mRCCD.jl:64-65,171,175,185) reaches ~1e-8 Eh
    w = make_named("S25").wfn()
    ints = ccd.make_rccd_integrals(w)
    e64 = ccd.do_rccd(w, maxit=60, r_conv=1e-11, integrals=ints)
    e32 = ccd.do_rccd(w, maxit=60, r_conv=1e-7, integrals=ints, diis_dtype=np.float32)
    assert abs(e64 - e32) < 1e-7


def test_ccsd_forms_agree_and_fae_variant_is_negligible():
    w = make_named("S25").wfn()
    e_jl = ccsd.do_rccsd(w, form="jl", maxit=40)
    e_m_textbook = ccsd.do_rccsd(w, form="m", fae_variant="jl", maxit=40)
    e_m_ref = ccsd.do_rccsd(w, form="m", maxit=40)
    assert abs(e_jl - e_m_textbook) < 1e-13
    assert abs(e_jl - e_m_ref) < 1e-11


def test_synthetic_generator_is_deterministic_and_symmetric():
    a = make_system(12, 3, 36, seed=11)
    b = make_system(12, 3, 36, seed=11)
    assert np.array_equal(a.B, b.B) and np.array_equal(a.C, b.C)
    g = a.ao_eri()
    assert np.allclose(g, np.transpose(g, (1, 0, 2, 3)))
    assert np.allclose(g, np.transpose(g, (2, 3, 0, 1)))
    assert np.allclose(a.C.T @ a.C, np.eye(12), atol=1e-13)
    assert np.all(np.diff(a.eps[:3]) >= 0) and np.all(np.diff(a.eps[3:]) >= 0)


def test_df_rmp2_oracle_equals_conventional_on_exact_factorisation():
    # the synthetic integrals are exactly B^T B, so DF-MP2 (DF-RMP2.jl:1-46) with b = B,
    # or with b hidden behind an orthogonal J^-1/2, equals conventional MP2
    s = make_named("S25")
    w = s.wfn()
    b = np.transpose(s.B, (1, 2, 0))
    e = oracle.do_rmp2(w)
    assert abs(oracle.df_rmp2(w, b) - e) < 1e-12
    Q, _ = np.linalg.qr(np.random.default_rng(7).standard_normal((s.naux, s.naux)))
    pqP = np.einsum("pqQ,PQ->pqP", b, Q)
    assert abs(oracle.df_rmp2(w, pqP, Q) - e) < 1e-12
