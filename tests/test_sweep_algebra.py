"""The device CCD sweep's contraction sequence, restated in numpy, against the reference's
equations (no GPU).

`ccd_sweep` (csrc/cc.cu) does not evaluate RCCD.jl's T2 update term by term: Wabef is never
formed, the (i,a)<->(j,b) image terms go through one Z array that the finalisation
symmetrises, the two Fmi terms ride in the hole-hole ladder, Fmi and Fae are traces of the
hole-hole and ring intermediates, the Z.Fae term rides in the first ring GEMM, and the energy is
one dot product with precomputed weights.  Each GETT below is one device contraction, written
with the same operands and index roles; the result must equal RCCD.jl's einsum form
(oracle.ccd.jl_cciter) and the reference energy to rounding.
"""
import numpy as np

from oracle import ccd
from oracle.mp2 import denominators
from juesgpu.synthetic import make_named

E = lambda s, *ops: np.einsum(s, *ops, optimize=True)  # noqa: E731


def device_form_sweep(T, oovv, vvvv, oooo, ovov, ovvo, D, df_wmbej=False, parts=None):
    o = T.shape[0]
    oovvT = 2.0 * oovv - oovv.transpose(1, 0, 2, 3)               # energy weights, formed once
    X = E("mnef,ijef->mnij", oovv, T)                             # ccd_x: W' = oooo + X
    Wp = oooo + X
    Fmi = 2.0 * np.einsum("mnin->mi", X) - np.einsum("mnni->mi", X)   # fmi_from_x
    d = np.eye(o)
    Wp = Wp - E("mi,nj->mnij", d, Fmi) - E("nj,mi->mnij", d, Fmi)  # wp_fmi: the two Fmi terms
    L = oovv + E("mnij,mnab->ijab", Wp, T) + E("ijef,abef->ijab", T, vvvv)   # hh and pp ladders
    J0 = ovvo                                                     # ring seeds
    K0 = -ovov.transpose(0, 1, 3, 2)
    # ccd_wj x2, ccd_wk: T read as T[j,n,b,f] and T[n,j,b,f] (the ring GEMMs' two A layouts)
    WJ = (J0 + 0.5 * E("mnef,jnbf->mbej", oovv if df_wmbej else oovvT, T)
          - 0.5 * E("mnef,njbf->mbej", oovv, T))
    WK = K0 + 0.5 * E("nmef,njbf->mbej", oovv, T)
    W12 = 2.0 * WJ + WK                                           # axpby
    tJ = np.einsum("maem->ae", WJ - J0)                           # fae_from_rings: traces over m
    tK = np.einsum("maem->ae", WK - K0)
    Fae = -2.0 * (tJ + tK) if df_wmbej else -(tJ + 2.0 * tK)
    for j in range(o):
        W12[j, :, :, j] += Fae                                    # W12[j,b,e,j] += Fae[b,e]
    Z = (E("imae,mbej->ijab", T, W12)                             # ccd_ring x3
         - E("miae,mbej->ijab", T, WJ)
         + E("mibe,maej->ijab", T, WK))
    if parts is not None:
        parts.update(Fae=Fae, Fmi=Fmi, WJ=WJ, WK=WK)
    return (L + Z + Z.transpose(1, 0, 3, 2)) / D                  # t2_finalize


def energy_device_form(T, oovv):
    return float(np.sum(T * (2.0 * oovv - oovv.transpose(1, 0, 2, 3))))


def test_device_sweep_equals_reference_update():
    s = make_named("S25")
    w = s.wfn()
    oovv, ovov, ovvo, oooo, vvvv = ccd.make_rccd_integrals(w)
    D = denominators(w.epsa, w.nalpha)
    # MP2 amplitudes, then one reference sweep: a pair-symmetric T that is not a fixed point
    T0 = oovv / D
    T = ccd.jl_cciter(T0, oovv, vvvv, oooo, ovov, ovvo, D)
    assert np.abs(T - T.transpose(1, 0, 3, 2)).max() < 1e-14
    ref = ccd.jl_cciter(T, oovv, vvvv, oooo, ovov, ovvo, D)
    dev = device_form_sweep(T, oovv, vvvv, oooo, ovov, ovvo, D)
    assert np.abs(dev - ref).max() < 1e-12 * np.abs(ref).max()
    assert abs(energy_device_form(T, oovv) - ccd.ccenergy(T, oovv)) < 1e-13 * abs(ccd.ccenergy(T, oovv))


def test_trace_forms_of_fae_fmi_and_ring_layouts():
    # the intermediates of the device form against RCCD.jl's own expressions (RCCD.jl:179, 216,
    # 400, 445) and, for df_wmbej, DF-RCCD.jl:239-242's WmBeJ, on a pair-symmetric T
    s = make_named("S25")
    w = s.wfn()
    oovv, ovov, ovvo, oooo, vvvv = ccd.make_rccd_integrals(w)
    D = denominators(w.epsa, w.nalpha)
    T = ccd.jl_cciter(oovv / D, oovv, vvvv, oooo, ovov, ovvo, D)
    Tt = 2.0 * T - T.transpose(1, 0, 2, 3)
    scale = np.abs(oovv).max() * np.abs(T).max() * T.size ** 0.5
    for df in (False, True):
        p = {}
        device_form_sweep(T, oovv, vvvv, oooo, ovov, ovvo, D, df_wmbej=df, parts=p)
        last = "mnef,njfb->mbej" if df else "nmef,njfb->mbej"
        WJ = ovvo + 0.5 * E("mnef,njfb->mbej", oovv, Tt) - 0.5 * E(last, oovv, T)
        WK = -ovov.transpose(0, 1, 3, 2) + 0.5 * E("jnfb,nmef->mbej", T, oovv)
        assert np.abs(p["WJ"] - WJ).max() < 1e-14 * scale
        assert np.abs(p["WK"] - WK).max() < 1e-14 * scale
        assert np.abs(p["Fae"] + E("mnaf,mnef->ae", Tt, oovv)).max() < 1e-14 * scale
        assert np.abs(p["Fmi"] - E("mnef,inef->mi", oovv, Tt)).max() < 1e-14 * scale


def test_ccsd_wabef_t1_terms_through_y():
    # ccsd_sweep never forms Wabef: its t1 parts, sum_ef Ttau[ij,ef] (-t1[m,b] <am|ef> - t1[m,a]
    # <mb|ef>), become -sum_m t1[m,b] Y[ij,a,m] with Y = Ttau . <am|ef>, plus its (i,a)<->(j,b)
    # image, which the finalisation adds (Z[i,j,a,b] + Z[j,i,b,a]).  On real integrals and a
    # pair-symmetric Ttau the two agree to rounding.
    from oracle import ccsd
    w = make_named("S25").wfn()
    oooo, ooov, oovv, ovov, ovvv, vvvv = ccsd.make_rccsd_integrals(w)
    o, v = w.nalpha, oovv.shape[2]
    rng = np.random.default_rng(3)
    t1 = 0.05 * rng.normal(size=(o, v))
    T2 = 0.05 * rng.normal(size=(o, o, v, v))
    T2 = 0.5 * (T2 + T2.transpose(1, 0, 3, 2))                       # pair symmetry
    Ttau = T2 + E("ia,jb->ijab", t1, t1)
    # the reference's form: Wabef's t1 parts (<am|ef> = ovvv[m,a,f,e], <mb|ef> = ovvv[m,b,e,f])
    W1 = -E("mb,mafe->abef", t1, ovvv) - E("ma,mbef->abef", t1, ovvv)
    ref = E("ijef,abef->ijab", Ttau, W1)
    # the device form: ccsd_y then ccsd_y_t1 into Z, symmetrised by t2_finalize
    Y = E("ijef,mafe->ijam", Ttau, ovvv)
    Z = -E("ijam,mb->ijab", Y, t1)
    dev = Z + Z.transpose(1, 0, 3, 2)
    assert np.abs(dev - ref).max() < 1e-14 * max(1.0, np.abs(ref).max())


def ccsd_device_form(blocks, t1, T, variant="jl", fock=None):
    """ccsd_sweep's sequence (csrc/cc.cu) in numpy: returns (R1, the T2 numerator).

    Fme from oovvT; Fmi from the trace of X = oovv . Ttau^T; the T2 parts of WmBeJ / WmBEj as
    three GEMMs on T2 and U = T2 + 2 tau; Fae, H1, G2 from the traces of WJ and WK before and
    after their t1 terms; T1's <ma|fe> terms from the traces of Y; F~ae in the first ring GEMM,
    F~mi in the hole-hole ladder with the rank-one correction t1[i,a] q[b,j] in the finalisation;
    Z's t1 terms with t1 on b (Wabef's, the two tau terms, the ooov term) as one -Q . t1.
    """
    oooo, ooov, oovv, ovov, ovvv, vvvv = blocks
    o, v = t1.shape
    W = oovv
    oovvT = 2 * W - W.transpose(1, 0, 2, 3)
    ooovT = 2 * ooov - ooov.transpose(1, 0, 2, 3)
    c1 = np.einsum("nmme->ne", ooov)
    c2 = np.einsum("mnme->ne", ooov)
    J0 = oovv.transpose(0, 3, 2, 1)
    K0 = -ovov.transpose(0, 1, 3, 2)
    tt = E("ma,nf->mnaf", t1, t1)
    Ttau, U = T + tt, T + 2 * tt                                        # ccsd_tau
    Fme = E("nf,mnef->me", t1, oovvT)                                   # ccsd_fme
    X = E("mnef,ijef->mnij", W, Ttau)                                   # ccsd_x
    Wp = oooo + X
    Fmi = 2 * np.einsum("mnin->mi", X) - np.einsum("mnni->mi", X) - 0.5 * E("me,ie->mi", Fme, t1)
    Fmi += 2 * E("ne,mnie->mi", t1, ooov) - E("ne,nmie->mi", t1, ooov)   # ccsd_fmi_t1
    Wp += E("je,mnie->mnij", t1, ooov) + E("ie,nmje->mnij", t1, ooov)     # ccsd_wmnij_t1
    fOV = np.zeros((o, v))
    if fock is not None:
        fOO, fOV, fVV = fock
        Fmi = Fmi + fOO + 0.5 * E("me,ie->mi", fOV, t1)
        Fme = Fme + fOV
    Fmt = Fmi + 0.5 * E("me,je->mj", Fme, t1)                           # ccsd_ftilde
    d = np.eye(o)
    Wp = Wp - E("mi,nj->mnij", d, Fmt) - E("nj,mi->mnij", d, Fmt)       # wp_fmi
    L = oovv + E("mnij,mnab->ijab", Wp, Ttau) + E("ijef,abef->ijab", Ttau, vvvv)
    WJ = J0 + 0.5 * E("mnef,jnbf->mbej", oovvT, T) - 0.5 * E("mnef,njbf->mbej", W, U)
    WK = K0 + 0.5 * E("nmef,njbf->mbej", W, U)
    tGJ, tGK = np.einsum("maem->ae", WJ - J0), np.einsum("maem->ae", WK - K0)   # ring_traces
    WJ = WJ + E("jf,mbef->mbej", t1, ovvv) - E("nb,nmje->mbej", t1, ooov)
    WK = WK - E("jf,mbfe->mbej", t1, ovvv) + E("nb,mnje->mbej", t1, ooov)
    W12 = 2 * WJ + WK
    # ccsd_fae_kernel
    H1 = np.einsum("maem->ae", WJ - J0) - tGJ + E("na,ne->ae", t1, c1)
    G2 = tGK - np.einsum("maem->ae", WK - K0) + E("na,ne->ae", t1, c2)
    Ft = 2 * G2 - (H1.T if variant == "m" else H1) - (tGJ + 2 * tGK) - E("ma,me->ae", t1, fOV)
    if fock is not None:
        Ft = Ft + fock[2]
    Fae = Ft + 0.5 * E("ma,me->ae", t1, Fme)
    for j in range(o):
        W12[j, :, :, j] += Ft
    # ccsd_y, seeded with ooov[m,i,j,a] at [(i,j),(a,m)]
    Y = E("ijef,mafe->ijam", Ttau, ovvv) + ooov.transpose(1, 2, 3, 0)
    c2 = np.einsum("mima->ia", ooov)                                    # the seed's two traces
    c3 = np.einsum("mmia->ia", ooov)
    R1 = (E("ie,ae->ia", t1, Fae) - E("ma,mi->ia", t1, Fmi)
          + 2 * E("me,imae->ia", Fme, T) - E("me,miae->ia", Fme, T)
          + 2 * E("me,imae->ia", t1, oovv) - E("me,maie->ia", t1, ovov)
          - E("mnae,mnie->ia", T, ooovT))
    R1 += (2 * (np.einsum("imam->ia", Y) - c2 - E("ie,ae->ia", t1, G2))
           - (np.einsum("miam->ia", Y) - c3 - E("if,af->ia", t1, H1)))   # t1_ytrace
    # Q[i,j,a,m] = Y (with its ooov seed) + Y1[j,m,i,a] + Y2[i,m,a,j] (the t1-on-b terms, imaged)
    Y1 = E("ie,mjeb->imjb", t1, oovv)
    Y2 = E("ie,maje->imaj", t1, ovov)
    Q = Y + Y1.transpose(2, 0, 3, 1) + Y2.transpose(0, 3, 2, 1)
    Z = (E("imae,mbej->ijab", T, W12) - E("miae,mbej->ijab", T, WJ) + E("mibe,maej->ijab", T, WK)
         - E("ijam,mb->ijab", Q, t1) + E("ie,jabe->ijab", t1, ovvv))
    if fock is not None:
        R1 = R1 + fOV
    q = E("mb,mj->bj", t1, Fmt)
    C = E("ia,bj->ijab", t1, q)
    return R1, L + Z + Z.transpose(1, 0, 3, 2) + C + C.transpose(1, 0, 3, 2)


def test_ccsd_device_form_equals_reference_update():
    # mRCCSD.jl:118-241 (oracle.ccsd.m_cciter) with the Fae t1 term of RCCSD.jl:190 ("jl") and of
    # mRCCSD.jl:140 ("m"), on a pair-symmetric T2 from one reference sweep
    from oracle import ccsd
    w = make_named("S25").wfn()
    blocks = ccsd.make_rccsd_integrals(w)
    o, v = w.nalpha, blocks[2].shape[2]
    eps = w.epsa
    D = denominators(eps, o)
    Dia = eps[:o, None] - eps[None, o:o + v]
    rng = np.random.default_rng(3)
    t1, T2 = ccsd.m_cciter(blocks, 0.05 * rng.normal(size=(o, v)), blocks[2] / D, Dia, D, fae_variant="jl")
    assert np.abs(T2 - T2.transpose(1, 0, 3, 2)).max() < 1e-15
    for variant in ("jl", "m"):
        r1, r2 = ccsd.m_cciter(blocks, t1, T2, Dia, D, fae_variant=variant)
        d1, d2 = ccsd_device_form(blocks, t1, T2, variant)
        assert np.abs(d1 / Dia - r1).max() < 1e-13 * np.abs(r1).max()
        assert np.abs(d2 / D - r2).max() < 1e-13 * np.abs(r2).max()


def test_ccsd_device_form_fock_terms():
    # the non-canonical Fock terms (Fae += f_ae - 1/2 t1^T f_ov, Fmi += f_mi + 1/2 f_ov t1^T,
    # Fme += f_ov, R1 += f_ov) through the trace forms, against the same terms added to the
    # reference intermediates (oracle.ccsd m_* functions)
    from oracle import ccsd
    w = make_named("S25").wfn()
    blocks = ccsd.make_rccsd_integrals(w)
    oooo, ooov, oovv, ovov, ovvv, vvvv = blocks
    o, v = w.nalpha, oovv.shape[2]
    rng = np.random.default_rng(8)
    t1 = 0.05 * rng.normal(size=(o, v))
    T2 = 0.05 * rng.normal(size=(o, o, v, v))
    T2 = 0.5 * (T2 + T2.transpose(1, 0, 3, 2))
    fOO = 0.01 * rng.normal(size=(o, o)); fOO = fOO + fOO.T; np.fill_diagonal(fOO, 0.0)
    fVV = 0.01 * rng.normal(size=(v, v)); fVV = fVV + fVV.T; np.fill_diagonal(fVV, 0.0)
    fOV = 0.01 * rng.normal(size=(o, v))
    tt = ccsd.tau(t1)
    Fae = ccsd.m_Fae(ovvv, oovv, t1, tt, T2, "jl") + fVV - 0.5 * E("ma,me->ae", t1, fOV)
    Fmi = ccsd.m_Fmi(ooov, oovv, t1, tt, T2) + fOO + 0.5 * E("me,ie->mi", fOV, t1)
    Fme = ccsd.m_Fme(oovv, t1) + fOV
    ones = np.ones((o, v))
    r1 = ccsd.m_T1(Fae, Fmi, Fme, oovv, ovov, ooov, ovvv, t1, T2, ones) + fOV
    Wabef = ccsd.m_Wabef(vvvv, ovvv, oovv, t1, tt, T2)
    Wmnij = ccsd.m_Wmnij(oooo, ooov, oovv, t1, tt, T2)
    WJ = ccsd.m_WmBeJ(ovvv, ooov, oovv, t1, tt, T2)
    WK = ccsd.m_WmBEj(ovov, ovvv, ooov, oovv, t1, tt, T2)
    r2 = ccsd.m_T2(Fae, Fmi, Fme, Wabef, Wmnij, WJ, WK, oovv, ovov, ovvv, ooov, t1, tt, T2,
                   np.ones_like(T2))
    d1, d2 = ccsd_device_form(blocks, t1, T2, "jl", fock=(fOO, fOV, fVV))
    assert np.abs(d1 - r1).max() < 1e-13 * np.abs(r1).max()
    assert np.abs(d2 - r2).max() < 1e-13 * np.abs(r2).max()
