"""Closed-shell CCSD (oracle; test infrastructure).

Two restatements of the reference:

* ``src/CoupledCluster/mRCCSD.jl`` (6 physicists' blocks from get_eri with
  lower-case specs, :102-110; intermediates :137-201; T1 :202-212; T2
  :213-241; energy :111-117; driver :35-101), and
* ``src/CoupledCluster/RCCSD.jl`` (15 blocks from tei_transform, :117-142;
  intermediates :187-247; T1 :248-259; T2 :260-289).

They agree everywhere except the t1 term of Fae: mRCCSD.jl:140 contracts
t[m,f] with ovvv[m,e,a,f] = <me|af> where RCCSD.jl:190 (and the textbook
closed-shell equations) use <ma|ef>.  ``fae_variant`` selects which.
"""
import numpy as np

from .jl import gemm, jperm, jreshape
from .mp2 import denominators
from .transform import get_eri, tei_transform

E = lambda s, *ops: np.einsum(s, *ops, optimize=True)  # noqa: E731


def make_rccsd_integrals(wfn):
    """mRCCSD.jl:102-110."""
    return tuple(get_eri(wfn, s) for s in ("oooo", "ooov", "oovv", "ovov", "ovvv", "vvvv"))


def make_rccsd_integrals_jl(gao, Cao, Cav):
    """RCCSD.jl:117-142, returned as a dict keyed by the reference's names."""
    O, V = Cao, Cav
    p = (0, 2, 1, 3)
    tt = lambda a, b, c, d: np.transpose(tei_transform(gao, a, b, c, d), p)  # noqa: E731
    blk = dict(vvvv=tt(V, V, V, V), ovvv=tt(O, V, V, V), vovv=tt(V, V, O, V),
               vvov=tt(V, O, V, V), vvvo=tt(V, V, V, O), oovv=tt(O, V, O, V),
               ovvo=tt(O, V, V, O), vovo=tt(V, V, O, O), ovov=tt(O, O, V, V),
               voov=tt(V, O, O, V), ooov=tt(O, O, O, V), oovo=tt(O, V, O, O),
               ovoo=tt(O, O, V, O), vooo=tt(V, O, O, O), oooo=tt(O, O, O, O))
    blk["vvov"] = jperm(blk["vvov"], 4, 1, 2, 3)     # :133
    blk["vvvo"] = jperm(blk["vvvo"], 3, 1, 2, 4)     # :134
    blk["vovv"] = jperm(blk["vovv"], 2, 1, 3, 4)     # :135
    blk["vooo"] = jperm(blk["vooo"], 2, 1, 3, 4)     # :136
    return blk


def tau(t1):
    """tiatia[m,n,a,f] = t1[m,a] t1[n,f] (mRCCSD.jl:70-72,86-88)."""
    return E("ma,nf->mnaf", t1, t1)


def ccenergy(oovv, t1, tt, T2):
    """mRCCSD.jl:111-117 / RCCSD.jl:143-149."""
    return float(np.sum(oovv * (2 * T2 + 2 * tt - np.transpose(T2, (1, 0, 2, 3))
                                - np.transpose(tt, (1, 0, 2, 3)))))


# --------------------------------------------------------------------------
# 6-block form (mRCCSD.jl)
# --------------------------------------------------------------------------
def m_Fae(ovvv, oovv, t1, tt, T2, fae_variant="m"):     # mRCCSD.jl:137-149
    o, v = T2.shape[0], T2.shape[2]
    if fae_variant == "m":
        ov3 = (2 * jreshape(jperm(ovvv, 1, 3, 2, 4), o * v, v * v)
               - jreshape(jperm(ovvv, 1, 4, 3, 2), o * v, v * v))
    else:   # <ma|ef> as RCCSD.jl:190
        ov3 = (2 * jreshape(jperm(ovvv, 1, 3, 2, 4), o * v, v * v)
               - jreshape(jperm(ovvv, 1, 4, 2, 3), o * v, v * v))
    Fae = jreshape(gemm("N", "N", 1.0, jreshape(t1, 1, o * v), ov3, 0.0, None), v, v)
    t = (jreshape(jperm(T2, 3, 1, 2, 4), v, o * o * v)
         + 0.5 * jreshape(jperm(tt, 3, 1, 2, 4), v, o * o * v))
    m = (2 * jreshape(jperm(oovv, 1, 2, 4, 3), o * o * v, v)
         - jreshape(jperm(oovv, 2, 1, 4, 3), o * o * v, v))
    return gemm("N", "N", -1.0, t, m, 1.0, Fae)


def m_Fmi(ooov, oovv, t1, tt, T2):                       # mRCCSD.jl:150-162
    o, v = T2.shape[0], T2.shape[2]
    oo3 = (2 * jreshape(jperm(ooov, 2, 4, 1, 3), o * v, o * o)
           - jreshape(jperm(ooov, 1, 4, 2, 3), o * v, o * o))
    Fmi = jreshape(gemm("N", "N", 1.0, jreshape(t1, 1, o * v), oo3, 0.0, None), o, o)
    m = 2 * jreshape(oovv, o, v * v * o) - jreshape(jperm(oovv, 1, 2, 4, 3), o, v * v * o)
    t = (jreshape(jperm(T2, 2, 3, 4, 1), v * v * o, o)
         + 0.5 * jreshape(jperm(tt, 2, 3, 4, 1), v * v * o, o))
    return gemm("N", "N", 1.0, m, t, 1.0, Fmi)


def m_Fme(oovv, t1):                                     # mRCCSD.jl:163-168
    return E("nf,mnef->me", t1, 2 * oovv - np.transpose(oovv, (1, 0, 2, 3)))


def m_Wmnij(oooo, ooov, oovv, t1, tt, T2):               # mRCCSD.jl:169-176
    return (oooo + E("je,mnie->mnij", t1, ooov) + E("ie,nmje->mnij", t1, ooov)
            + 0.5 * E("ijef,mnef->mnij", T2 + tt, oovv))


def m_Wabef(vvvv, ovvv, oovv, t1, tt, T2):               # mRCCSD.jl:177-184
    return (vvvv - E("mb,mafe->abef", t1, ovvv) - E("ma,mbef->abef", t1, ovvv)
            + 0.5 * E("mnab,mnef->abef", T2 + tt, oovv))


def m_WmBeJ(ovvv, ooov, oovv, t1, tt, T2):               # mRCCSD.jl:185-193
    return (np.transpose(oovv, (0, 3, 2, 1)) + E("jf,mbef->mbej", t1, ovvv)
            - E("nb,nmje->mbej", t1, ooov)
            - 0.5 * E("jnfb,mnef->mbej", T2 + 2 * tt, oovv)
            + 0.5 * E("njfb,mnef->mbej", T2, 2 * oovv - np.transpose(oovv, (1, 0, 2, 3))))


def m_WmBEj(ovov, ovvv, ooov, oovv, t1, tt, T2):         # mRCCSD.jl:194-201
    return (-np.transpose(ovov, (0, 1, 3, 2)) - E("jf,mbfe->mbej", t1, ovvv)
            + E("nb,mnje->mbej", t1, ooov)
            + E("jnfb,nmef->mbej", 0.5 * T2 + tt, oovv))


def m_T1(Fae, Fmi, Fme, oovv, ovov, ooov, ovvv, t1, T2, Dia):   # mRCCSD.jl:202-212
    r = (E("ie,ae->ia", t1, Fae) - E("ma,mi->ia", t1, Fmi)
         + E("me,imae->ia", Fme, 2 * T2 - np.transpose(T2, (1, 0, 2, 3)))
         + E("me,imae->ia", t1, 2 * oovv) - E("me,maie->ia", t1, ovov)
         - E("mnae,mnie->ia", T2, 2 * ooov - np.transpose(ooov, (1, 0, 2, 3)))
         + E("imef,mafe->ia", T2, 2 * ovvv) - E("imef,maef->ia", T2, ovvv))
    return r / Dia


def m_T2(Fae, Fmi, Fme, Wabef, Wmnij, WmBeJ, WmBEj, oovv, ovov, ovvv, ooov,
         t1, tt, T2, D):                                          # mRCCSD.jl:213-241
    Tt = np.transpose
    r = (oovv
         + E("ijae,be->ijab", T2, Fae - 0.5 * E("mb,me->be", t1, Fme))
         + E("ijeb,ae->ijab", T2, Fae - 0.5 * E("ma,me->ae", t1, Fme))
         - E("imab,mj->ijab", T2, Fmi + 0.5 * E("je,me->mj", t1, Fme))
         - E("mjab,mi->ijab", T2, Fmi + 0.5 * E("ie,me->mi", t1, Fme))
         + E("mnab,mnij->ijab", T2 + tt, Wmnij)
         + E("ijef,abef->ijab", T2 + tt, Wabef)
         + E("imae,mbej->ijab", T2 - Tt(T2, (1, 0, 2, 3)), WmBeJ)
         - E("imea,mjeb->ijab", tt, oovv)
         + E("imae,mbej->ijab", T2, WmBeJ + WmBEj)
         + E("mibe,maej->ijab", T2, WmBEj) - E("imeb,maje->ijab", tt, ovov)
         + E("mjae,mbei->ijab", T2, WmBEj) - E("jmea,mbie->ijab", tt, ovov)
         + E("jmbe,maei->ijab", T2 - Tt(T2, (1, 0, 2, 3)), WmBeJ)
         - E("jmeb,miea->ijab", tt, oovv)
         + E("jmbe,maei->ijab", T2, WmBeJ + WmBEj)
         + E("ie,jabe->ijab", t1, ovvv) + E("je,ibae->ijab", t1, ovvv)
         - E("ma,mjib->ijab", t1, ooov) - E("mb,jima->ijab", t1, ooov))
    return r / D


def m_cciter(blocks, t1, T2, Dia, D, fae_variant="m"):          # mRCCSD.jl:118-135
    oooo, ooov, oovv, ovov, ovvv, vvvv = blocks
    tt = tau(t1)
    Fae = m_Fae(ovvv, oovv, t1, tt, T2, fae_variant)
    Fmi = m_Fmi(ooov, oovv, t1, tt, T2)
    Fme = m_Fme(oovv, t1)
    Wabef = m_Wabef(vvvv, ovvv, oovv, t1, tt, T2)
    Wmnij = m_Wmnij(oooo, ooov, oovv, t1, tt, T2)
    WmBeJ = m_WmBeJ(ovvv, ooov, oovv, t1, tt, T2)
    WmBEj = m_WmBEj(ovov, ovvv, ooov, oovv, t1, tt, T2)
    t1n = m_T1(Fae, Fmi, Fme, oovv, ovov, ooov, ovvv, t1, T2, Dia)
    T2n = m_T2(Fae, Fmi, Fme, Wabef, Wmnij, WmBeJ, WmBEj, oovv, ovov, ovvv, ooov,
               t1, tt, T2, D)
    return t1n, T2n


# --------------------------------------------------------------------------
# 15-block form (RCCSD.jl)
# --------------------------------------------------------------------------
def jl_cciter(b, t1, T2, Dia, D):                                # RCCSD.jl:150-173
    tt = tau(t1)
    Tt = np.transpose
    mnef = b["oovv"]
    Fae = (E("mf,maef->ae", t1, 2 * b["vovv"]) - E("mf,maef->ae", t1, b["ovvv"])
           - E("mnaf,mnef->ae", T2 + 0.5 * tt, 2 * mnef - Tt(mnef, (1, 0, 2, 3))))   # :187-194
    Fmi = (E("ne,mnie->mi", t1, 2 * b["ooov"] - Tt(b["ooov"], (1, 0, 2, 3)))
           + E("inef,mnef->mi", T2 + 0.5 * tt, 2 * mnef - Tt(mnef, (0, 1, 3, 2))))   # :195-203
    Fme = E("nf,mnef->me", t1, 2 * mnef - Tt(mnef, (1, 0, 2, 3)))                   # :204-210
    Wmnij = (b["oooo"] + E("je,mnie->mnij", t1, b["ooov"]) + E("ie,mnej->mnij", t1, b["oovo"])
             + 0.5 * E("ijef,mnef->mnij", T2 + tt, mnef))                          # :211-219
    Wabef = (b["vvvv"] - E("mb,maef->abef", t1, b["vovv"]) - E("ma,mbef->abef", t1, b["ovvv"])
             + 0.5 * E("mnab,mnef->abef", T2 + tt, mnef))                          # :220-228
    WmBeJ = (b["ovvo"] + E("jf,mbef->mbej", t1, b["ovvv"]) - E("nb,mnej->mbej", t1, b["oovo"])
             - 0.5 * E("jnfb,mnef->mbej", T2 + 2 * tt, mnef)
             + 0.5 * E("njfb,mnef->mbej", T2, 2 * mnef - Tt(mnef, (1, 0, 2, 3))))   # :229-238
    WmBEj = (-Tt(b["vovo"], (1, 0, 2, 3)) - E("jf,mbfe->mbej", t1, b["ovvv"])
             + E("nb,nmej->mbej", t1, b["oovo"])
             + E("jnfb,nmef->mbej", 0.5 * T2 + tt, mnef))                           # :239-247
    amie, maie, mnie, amef = b["voov"], b["ovov"], b["ooov"], b["vovv"]
    t1n = (E("ie,ae->ia", t1, Fae) - E("ma,mi->ia", t1, Fmi)
           + E("me,imae->ia", Fme, 2 * T2 - Tt(T2, (1, 0, 2, 3)))
           + E("me,amie->ia", t1, 2 * amie) - E("me,maie->ia", t1, maie)
           - E("mnae,mnie->ia", T2, 2 * mnie - Tt(mnie, (1, 0, 2, 3)))
           + E("imef,maef->ia", T2, 2 * amef) - E("imef,mafe->ia", T2, amef)) / Dia  # :248-259
    mbej, amej, abej, abie, mbij, amij = (b["ovvo"], b["vovo"], b["vvvo"], b["vvov"],
                                          b["ovoo"], b["vooo"])
    r = (mnef
         + E("ijae,be->ijab", T2, Fae - 0.5 * E("mb,me->be", t1, Fme))
         + E("ijeb,ae->ijab", T2, Fae - 0.5 * E("ma,me->ae", t1, Fme))
         - E("imab,mj->ijab", T2, Fmi + 0.5 * E("je,me->mj", t1, Fme))
         - E("mjab,mi->ijab", T2, Fmi + 0.5 * E("ie,me->mi", t1, Fme))
         + E("mnab,mnij->ijab", T2 + tt, Wmnij)
         + E("ijef,abef->ijab", T2 + tt, Wabef)
         + E("imae,mbej->ijab", T2 - Tt(T2, (1, 0, 2, 3)), WmBeJ) - E("imea,mbej->ijab", tt, mbej)
         + E("imae,mbej->ijab", T2, WmBeJ + WmBEj)
         + E("mibe,maej->ijab", T2, WmBEj) - E("imeb,amej->ijab", tt, amej)
         + E("mjae,mbei->ijab", T2, WmBEj) - E("jmea,bmei->ijab", tt, amej)
         + E("jmbe,maei->ijab", T2 - Tt(T2, (1, 0, 2, 3)), WmBeJ) - E("jmeb,maei->ijab", tt, mbej)
         + E("jmbe,maei->ijab", T2, WmBeJ + WmBEj)
         + E("ei,eabj->ijab", t1.T, abej) + E("ej,eabi->ijab", t1.T, abie)
         - E("ma,mbij->ijab", t1, mbij) - E("mb,maij->ijab", t1, amij))            # :260-289
    return t1n, r / D


def do_rccsd(wfn, maxit=40, return_T=False, form="m", fae_variant=None, diis=False,
             max_diis=6, r_conv=None, e_conv=None, log=None, blocks=None):
    """mRCCSD.do_rccsd (mRCCSD.jl:35-101) / RCCSD.do_rccsd (RCCSD.jl:33-116).

    T1 = 0, T2 = oovv/D (:55-66), ``maxit`` sweeps; optional FP64 DIIS over the
    concatenated (T1, T2) vector and convergence tests (extensions: the
    reference always runs 40 sweeps).
    """
    o, eps = wfn.nalpha, wfn.epsa
    D = denominators(eps, o)
    Dia = eps[:o, None] - eps[None, o:]
    if form == "m":
        if blocks is None:
            blocks = make_rccsd_integrals(wfn)
        oovv = blocks[2]
        fv = "m" if fae_variant is None else fae_variant
        sweep = lambda t1, T2: m_cciter(blocks, t1, T2, Dia, D, fv)  # noqa: E731
    else:
        if blocks is None:
            blocks = make_rccsd_integrals_jl(wfn.ao_eri, wfn.Cao, wfn.Cav)
        oovv = blocks["oovv"]
        sweep = lambda t1, T2: jl_cciter(blocks, t1, T2, Dia, D)  # noqa: E731
    nv = oovv.shape[2]
    t1 = np.zeros((o, nv))
    T2 = oovv / D
    from .ccd import DIIS
    n1 = t1.size
    dii = DIIS(np.concatenate([t1.ravel(), T2.ravel()]), max_diis) if diis else None
    e_old = ccenergy(oovv, t1, tau(t1), T2)
    niter = 0
    for i in range(maxit):
        t1n, T2n = sweep(t1, T2)
        if dii is not None:
            x, rms = dii.push_extrapolate(np.concatenate([t1n.ravel(), T2n.ravel()]),
                                          np.concatenate([t1.ravel(), T2.ravel()]))
            t1, T2 = x[:n1].reshape(t1.shape), x[n1:].reshape(T2.shape)
        else:
            rms = float(np.sqrt(np.sum((t1n - t1) ** 2) + np.sum((T2n - T2) ** 2)))
            t1, T2 = t1n, T2n
        niter = i + 1
        e = ccenergy(oovv, t1, tau(t1), T2)
        if log is not None:
            log.append((niter, e, rms))
        done = (r_conv is not None or e_conv is not None)
        if r_conv is not None:
            done = done and rms < r_conv
        if e_conv is not None:
            done = done and abs(e - e_old) < e_conv
        e_old = e
        if done:
            break
    e = ccenergy(oovv, t1, tau(t1), T2)
    return (e, t1, T2, niter) if return_T else e
