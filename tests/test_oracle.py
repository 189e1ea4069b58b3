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


def test_df_rccd_oracle_forms():
    # DF-RCCD.jl on exactly factorised integrals: with RCCD.jl's WmBeJ it is the RCCD
    # iteration itself (MP2 guess, no DIIS), sweep by sweep; DF-RCCD.jl's own WmBeJ (its last
    # term contracts (me|nf) where RCCD.jl:400 has (ne|mf)) reaches a different fixed point
    from oracle import df_rccd
    s = make_named("S25")
    w = s.wfn()
    b = np.transpose(s.B, (1, 2, 0))
    log_df, log_ref, log_q = [], [], []
    df_rccd.do_df_rccd(w, b, maxit=6, variant="rccd", log=log_df)
    ccd.do_rccd(w, maxit=6, guess="mp2", diis=False, r_conv=None, log=log_ref)
    for (i1, e1), (i2, e2, _) in zip(log_df, log_ref):
        assert i1 == i2 and abs(e1 - e2) < 1e-13
    e_q = df_rccd.do_df_rccd(w, b, maxit=40, variant="reference", log=log_q)
    e_r = df_rccd.do_df_rccd(w, b, maxit=40, variant="rccd")
    assert abs(log_q[-1][1] - log_q[-2][1]) < 1e-10      # both converge within 40 sweeps
    assert abs(e_q - e_r) > 1e-6


def _spin_orbital_pT(w, t1, T2):
    """Independent spin-orbital (T) (the textbook connected/disconnected triples with
    antisymmetrised integrals) on converged closed-shell CCSD amplitudes."""
    from oracle.transform import tei_transform
    C = w.Ca if hasattr(w, "Ca") else np.hstack([w.Cao, w.Cav])
    n, o = C.shape[1], w.nalpha
    mo = tei_transform(w.ao_eri, C)                       # (pq|rs), spatial
    ns, no = 2 * n, 2 * o
    # spin orbitals: occupied first (alpha, beta interleaved), then virtuals
    spat = [p // 2 for p in range(2 * o)] + [o + p // 2 for p in range(2 * (n - o))]
    spin = [p % 2 for p in range(ns)]
    sp = np.array(spat)
    sg = np.array(spin)
    chem = mo[np.ix_(sp, sp, sp, sp)] * ((sg[:, None] == sg[None, :])[:, :, None, None]
                                         * (sg[:, None] == sg[None, :])[None, None, :, :])
    phys = np.transpose(chem, (0, 2, 1, 3))               # <pq|rs> = (pr|qs)
    anti = phys - np.transpose(phys, (0, 1, 3, 2))
    eps = np.array([w.epsa[s] for s in spat])
    nv = ns - no
    # amplitudes
    ts1 = np.zeros((no, nv))
    ts2 = np.zeros((no, no, nv, nv))
    for I in range(no):
        for A in range(nv):
            if sg[I] == sg[no + A]:
                ts1[I, A] = t1[sp[I], sp[no + A] - o]
    for I in range(no):
        for J in range(no):
            for A in range(nv):
                for B in range(nv):
                    i, j, a, b = sp[I], sp[J], sp[no + A] - o, sp[no + B] - o
                    val = 0.0
                    if sg[I] == sg[no + A] and sg[J] == sg[no + B]:
                        val += T2[i, j, a, b]
                    if sg[I] == sg[no + B] and sg[J] == sg[no + A]:
                        val -= T2[i, j, b, a]
                    ts2[I, J, A, B] = val
    O, V = slice(0, no), slice(no, ns)
    eo, ev = eps[:no], eps[no:]
    D = (eo[:, None, None, None, None, None] + eo[None, :, None, None, None, None]
         + eo[None, None, :, None, None, None] - ev[None, None, None, :, None, None]
         - ev[None, None, None, None, :, None] - ev[None, None, None, None, None, :])
    E = np.einsum
    # t_c without permutation: sum_e t_jk^ae <ei||bc> - sum_m t_im^bc <ma||jk>
    raw_c = E("jkae,eibc->ijkabc", ts2, anti[V, O, V, V]) - E("imbc,majk->ijkabc", ts2, anti[O, V, O, O])
    raw_d = E("ia,jkbc->ijkabc", ts1, anti[O, O, V, V])

    def P(x):
        # P(i/jk) P(a/bc)
        y = x - np.transpose(x, (1, 0, 2, 3, 4, 5)) - np.transpose(x, (2, 1, 0, 3, 4, 5))
        return y - np.transpose(y, (0, 1, 2, 4, 3, 5)) - np.transpose(y, (0, 1, 2, 5, 4, 3))
    tc = P(raw_c) / D
    td = P(raw_d) / D
    return float(np.sum(tc * D * (tc + td)) / 36.0)


def test_pT_oracle_equals_spin_orbital_triples_on_h2o():
    # compute_pT (PerturbativeTriples.jl:35-138) has no known answer in the reference's tests;
    # pin its closed-shell restatement against an independent spin-orbital (T) on the same
    # converged H2O/STO-3G CCSD amplitudes, and its vectorised energy loop against the scalar one
    from oracle import triples
    w = h2o()
    e, t1, T2, _ = ccsd.do_rccsd(w, return_T=True)
    assert abs(e - E_CCSD_H2O) < 1e-10
    oooo, ooov, oovv, ovov, ovvv, vvvv = ccsd.make_rccsd_integrals(w)
    Vvvvo, Vvooo, Vvovo = triples.integrals_from_cc(ovvv, ooov, oovv)
    o = w.nalpha
    args = (t1, T2, Vvvvo, Vvooo, Vvovo, w.epsa[:o], w.epsa[o:])
    e_t = triples.compute_pT(*args)
    assert abs(e_t - triples.compute_pT_loops(*args)) < 1e-15
    e_so = _spin_orbital_pT(w, t1, T2)
    assert e_t < 0 and abs(e_t - e_so) < 1e-12, (e_t, e_so)


def _h2o_rotated(scale, seed=3):
    """H2O/STO-3G with its occupied and virtual orbitals each mixed by exp(scale * A), A
    antisymmetric: a non-canonical but equivalent reference."""
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


def test_auto_rccsd_oracle_pins():
    # AutoRCCSD.jl restated: the canonical H2O energy is the reference's CCSD known answer, the
    # Fock matrix of the RHF orbitals is diagonal with the orbital energies, a rotation of the
    # occupied and of the virtual orbitals leaves the energy unchanged, and with one frozen
    # core orbital it equals the canonical CCSD of the active space
    from oracle import auto_rccsd
    w = _h2o_rotated(0.0)
    f = auto_rccsd.get_fock(w.Ca, w.Cao, w.ao_eri, w.hao)
    assert np.abs(np.diag(f) - w.epsa).max() < 1e-10
    assert np.abs(f - np.diag(np.diag(f))).max() < 1e-10
    e = auto_rccsd.do_rccsd(w)
    assert abs(e - E_CCSD_H2O) < 1e-9
    e_rot = auto_rccsd.do_rccsd(_h2o_rotated(0.1))
    assert abs(e_rot - e) < 1e-9
    e_fc = auto_rccsd.do_rccsd(w, fcn=1)
    import dataclasses
    act = dataclasses.replace(w, nalpha=w.nalpha - 1, nbeta=w.nalpha - 1, Cao=w.Cao[:, 1:], Cbo=w.Cao[:, 1:],
                              epsa=w.epsa[1:], epsb=w.epsa[1:])
    assert abs(e_fc - ccsd.do_rccsd(act, maxit=80, diis=True)) < 1e-9
    assert abs(e_fc - e) > 1e-5


def test_pipelined_sweep_is_the_reference_sweep():
    # the CPU baseline's staged sweep (oracle/sampled.py) does exactly RCCD.jl's arithmetic: 16
    # stages from the (ij|ab)/D guess equal one jl_cciter, and 32 stages two of them
    from oracle.df_blocks import rccd_blocks_from_B
    from oracle.sampled import PipelinedSweep
    s = make_named("S25")
    o = s.nocc
    oovv, ovov, ovvo, oooo, vvvv = rccd_blocks_from_B(s.B, s.C, o)
    ps = PipelinedSweep(oovv, ovov, ovvo, oooo, vvvv, s.eps, o, stages=16)
    D = oracle.mp2.denominators(s.eps, o)
    T = np.transpose(ovov, (0, 2, 1, 3)) / D
    for sweep in range(2):
        T = ccd.jl_cciter(T, oovv, vvvv, oooo, ovov, ovvo, D)
        ks = [ps.step()[0] for _ in range(16)]
        assert ks == list(range(16)) and ps.sweeps == sweep + 1
        assert np.abs(ps.T - T).max() < 1e-13 * np.abs(T).max()
        assert abs(ps.energy - ccd.ccenergy(T, oovv)) < 1e-13
