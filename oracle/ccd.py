"""Closed-shell CCD (oracle; test infrastructure).

Two independent restatements of the reference, kept separate on purpose so that
they check each other:

* the einsum form of ``src/CoupledCluster/RCCD.jl`` (intermediates :169-467,
  T2 update :234-303, energy :99-117, driver :33-83), and
* the explicit permutedims/reshape/gemm form of ``src/CoupledCluster/mRCCD.jl``
  (intermediates :265-488, T2 update :301-394, energy :129-137, DIIS :138-208,
  driver :38-118).

Integral blocks are physicists' notation, column-major meaning as in Julia:
``oovv[i,j,a,b] = <ij|ab>``, ``ovov[i,a,j,b] = <ia|jb>``, ``ovvo[i,a,b,j] = <ia|bj>``,
``oooo``, ``vvvv``.
"""
import numpy as np

from .jl import gemm, jperm, jreshape
from .mp2 import denominators
from .transform import get_eri, tei_transform

E = lambda s, *ops: np.einsum(s, *ops, optimize=True)  # noqa: E731


# --------------------------------------------------------------------------
# integrals
# --------------------------------------------------------------------------
def make_rccd_integrals_jl(gao, Cao, Cav):
    """RCCD.jl:85-97 (tei_transform + permutedims [1,3,2,4])."""
    oovv = tei_transform(gao, Cao, Cav, Cao, Cav)
    vvvv = tei_transform(gao, Cav, Cav, Cav, Cav)
    ovvo = tei_transform(gao, Cao, Cav, Cav, Cao)
    ovov = tei_transform(gao, Cao, Cao, Cav, Cav)
    oooo = tei_transform(gao, Cao, Cao, Cao, Cao)
    p = (0, 2, 1, 3)
    return (np.transpose(oovv, p), np.transpose(ovov, p), np.transpose(ovvo, p),
            np.transpose(oooo, p), np.transpose(vvvv, p))


def make_rccd_integrals(wfn):
    """mRCCD.jl:120-127: get_eri of OOVV, VVVV, OVVO, OVOV, OOOO (phys)."""
    oovv = get_eri(wfn, "OOVV")
    vvvv = get_eri(wfn, "VVVV")
    ovvo = get_eri(wfn, "OVVO")
    ovov = get_eri(wfn, "OVOV")
    oooo = get_eri(wfn, "OOOO")
    return oovv, ovov, ovvo, oooo, vvvv


def ccenergy(T, oovv):
    """RCCD.jl:99-117 / mRCCD.jl:129-137."""
    return float(np.sum(oovv * (2.0 * T - np.transpose(T, (1, 0, 2, 3)))))


# --------------------------------------------------------------------------
# einsum form (RCCD.jl)
# --------------------------------------------------------------------------
def jl_Fae(T, mnef):        # RCCD.jl:169-198
    return -E("mnef,mnaf->ae", mnef, 2 * T - np.transpose(T, (1, 0, 2, 3)))


def jl_Fmi(T, mnef):        # RCCD.jl:208-232
    return E("mnef,inef->mi", mnef, 2 * T - np.transpose(T, (0, 1, 3, 2)))


def jl_Wmnij(mnij, mnef, T):   # RCCD.jl:312-341
    return mnij + E("ijef,mnef->mnij", T, mnef) / 2


def jl_Wabef(abef, mnef, T):   # RCCD.jl:350-380
    return E("mnab,mnef->abef", T, mnef) / 2 + abef


def jl_WmBeJ(mbej, mnef, T):   # RCCD.jl:390-425
    return (mbej + E("mnef,njfb->mbej", mnef, 2 * T - np.transpose(T, (1, 0, 2, 3))) / 2
            - E("nmef,njfb->mbej", mnef, T) / 2)


def jl_WmBEj(nmef, mbje, T):   # RCCD.jl:436-467
    return -np.transpose(mbje, (0, 1, 3, 2)) + E("jnfb,nmef->mbej", T, nmef) / 2.0


def jl_T2(T, Fae, Fmi, WmBeJ, WmBEj, Wabef, Wmnij, ijab, D):   # RCCD.jl:234-303
    R = (ijab + E("ijae,be->ijab", T, Fae) + E("jibe,ae->ijab", T, Fae)
         - E("imab,mj->ijab", T, Fmi) - E("mjab,mi->ijab", T, Fmi)
         + E("mnab,mnij->ijab", T, Wmnij)
         + E("ijef,abef->ijab", T, Wabef)
         + E("imae,mbej->ijab", T, WmBeJ) * 2
         - E("miae,mbej->ijab", T, WmBeJ)
         + E("imae,mbej->ijab", T, WmBEj)
         + E("mibe,maej->ijab", T, WmBEj)
         + E("mjae,mbei->ijab", T, WmBEj)
         + E("jmbe,maei->ijab", T, WmBeJ) * 2
         - E("mjbe,maei->ijab", T, WmBeJ)
         + E("jmbe,maei->ijab", T, WmBEj))
    return R / D


def jl_cciter(T, oovv, vvvv, oooo, ovov, ovvo, D):   # RCCD.jl:119-143
    Wabef = jl_Wabef(vvvv, oovv, T)
    WmBeJ = jl_WmBeJ(ovvo, oovv, T)
    WmBEj = jl_WmBEj(oovv, ovov, T)
    Wmnij = jl_Wmnij(oooo, oovv, T)
    Fae = jl_Fae(T, oovv)
    Fmi = jl_Fmi(T, oovv)
    return jl_T2(T, Fae, Fmi, WmBeJ, WmBEj, Wabef, Wmnij, oovv, D)


def do_rccd_jl(wfn, maxit=40, return_T2=False, log=None):
    """RCCD.do_rccd (RCCD.jl:33-83): T2 init (ij|ab)/D, fixed maxit sweeps, no DIIS."""
    o, eps = wfn.nalpha, wfn.epsa
    oovv, ovov, ovvo, oooo, vvvv = make_rccd_integrals_jl(wfn.ao_eri, wfn.Cao, wfn.Cav)
    D = denominators(eps, o)
    T = np.transpose(ovov, (0, 2, 1, 3)) / D          # T2_init! :145-160
    for _ in range(maxit):
        T = jl_cciter(T, oovv, vvvv, oooo, ovov, ovvo, D)
        if log is not None:
            log.append(ccenergy(T, oovv))
    e = ccenergy(T, oovv)
    return (e, T) if return_T2 else e


# --------------------------------------------------------------------------
# GEMM form (mRCCD.jl)
# --------------------------------------------------------------------------
def m_Fae(T, mnef):          # mRCCD.jl:265-275
    o, v = T.shape[0], T.shape[2]
    t = 2 * jreshape(jperm(T, 3, 1, 2, 4), v, o * o * v)
    t = t - jreshape(jperm(T, 3, 2, 1, 4), v, o * o * v)
    m = jreshape(jperm(mnef, 1, 2, 4, 3), o * o * v, v)
    return gemm("N", "N", -1.0, t, m, 0.0, None)


def m_Fmi(T, mnef):          # mRCCD.jl:285-299
    o, v = T.shape[0], T.shape[2]
    t = 2 * jreshape(jperm(T, 2, 3, 4, 1), o * v * v, o)
    t = t - jreshape(jperm(T, 2, 4, 3, 1), o * v * v, o)
    m = jreshape(mnef, o, o * v * v)
    return gemm("N", "N", 1.0, m, t, 0.0, None)


def m_Wmnij(mnij, mnef, T):  # mRCCD.jl:403-415
    o, v = T.shape[0], T.shape[2]
    W = jreshape(mnij, o * o, o * o)
    W = gemm("N", "T", 0.5, jreshape(mnef, o * o, v * v), jreshape(T, o * o, v * v), 1.0, W)
    return jreshape(W, o, o, o, o)


def m_Wabef(abef, mnef, T):  # mRCCD.jl:424-436
    o, v = T.shape[0], T.shape[2]
    W = jreshape(abef, v * v, v * v)
    W = gemm("T", "N", 0.5, jreshape(T, o * o, v * v), jreshape(mnef, o * o, v * v), 1.0, W)
    return jreshape(W, v, v, v, v)


def m_WmBeJ(mbej, mnef, T):  # mRCCD.jl:446-464
    o, v = T.shape[0], T.shape[2]
    W = jreshape(jperm(mbej, 1, 3, 4, 2), o * v, o * v)
    t1 = 2 * jreshape(jperm(T, 1, 3, 2, 4), o * v, o * v) - jreshape(jperm(T, 2, 3, 1, 4), o * v, o * v)
    m1 = jreshape(jperm(mnef, 1, 3, 2, 4), o * v, o * v)
    m2 = jreshape(jperm(mnef, 1, 4, 2, 3), o * v, o * v)
    t2 = jreshape(jperm(T, 1, 3, 2, 4), o * v, o * v)
    W = gemm("N", "N", 0.5, m1, t1, 1.0, W)
    W = gemm("T", "N", -0.5, m2, t2, 1.0, W)
    return jperm(jreshape(W, o, v, o, v), 1, 4, 2, 3)


def m_WmBEj(nmef, mbje, T):  # mRCCD.jl:475-488
    o, v = T.shape[0], T.shape[2]
    W0 = -jperm(mbje, 1, 2, 4, 3)
    t = jreshape(jperm(T, 2, 3, 1, 4), o * v, o * v)
    m = jreshape(jperm(nmef, 2, 3, 1, 4), o * v, o * v)
    W = jreshape(jperm(W0, 1, 3, 4, 2), o * v, o * v)
    W = gemm("N", "N", 0.5, m, t, 1.0, W)
    return jperm(jreshape(W, o, v, o, v), 1, 4, 2, 3)


def m_T2(Ti, Fae, Fmi, WmBeJ, WmBEj, Wabef, Wmnij, ijab, D):   # mRCCD.jl:301-394
    o, v = ijab.shape[0], ijab.shape[2]
    ov = o * v
    d = ijab.copy()
    d = jreshape(gemm("N", "T", 1.0, jreshape(Ti, o * o * v, v), Fae, 1.0,
                      jreshape(d, o * o * v, v)), o, o, v, v)                      # :312-315
    x = jreshape(jperm(d, 2, 1, 4, 3), o * o * v, v)                              # :317-319
    x = gemm("N", "T", 1.0, jreshape(Ti, o * o * v, v), Fae, 1.0, x)              # :321
    d = jperm(jreshape(x, o, o, v, v), 2, 1, 4, 3)                                # :322
    x = jreshape(jperm(d, 1, 3, 4, 2), o * v * v, o)                              # :324-325
    ti = jreshape(jperm(Ti, 2, 1, 3, 4), o, o * v * v)                            # :326
    x = gemm("T", "N", -1.0, ti, Fmi, 1.0, x)                                     # :327
    d = jperm(jreshape(x.T, o, o, v, v), 2, 1, 3, 4)                              # :328
    x = jreshape(jperm(d, 2, 3, 4, 1), o * v * v, o)                              # :331-332
    x = gemm("T", "N", -1.0, jreshape(Ti, o, o * v * v), Fmi, 1.0, x)             # :333-334
    d = jreshape(x.T, o, o, v, v)                                                 # :335
    x = jreshape(d, o * o, v * v)
    tiv = jreshape(Ti, o * o, v * v)
    x = gemm("T", "N", 1.0, jreshape(Wmnij, o * o, o * o), tiv, 1.0, x)           # :340
    x = gemm("N", "T", 1.0, tiv, jreshape(Wabef, v * v, v * v), 1.0, x)           # :343
    d = jreshape(x, o, o, v, v)
    x = jreshape(jperm(d, 1, 3, 4, 2), ov, ov)                                    # :351-352
    scr2 = jreshape(jperm(Ti, 1, 3, 2, 4), ov, ov)                                # :353-354
    scr3 = 2 * jreshape(jperm(WmBeJ, 1, 3, 2, 4), ov, ov)                         # :355-356
    itm = jreshape(jperm(WmBEj, 1, 3, 2, 4), ov, ov)                              # :358-359
    scr3 = scr3 + itm                                                             # :360
    x = gemm("N", "N", 1.0, scr2, scr3, 1.0, x)                                   # :361
    scr3 = (scr3 - itm) * 0.5                                                     # :363-364
    scr2 = jreshape(jperm(Ti, 1, 4, 2, 3), ov, ov)                                # :365
    x = gemm("T", "N", -1.0, scr2, scr3, 1.0, x)                                  # :366
    d = jperm(jreshape(x, o, v, v, o), 1, 4, 2, 3)                                # :368
    x = jreshape(jperm(d, 1, 4, 3, 2), ov, ov)                                    # :370
    scr2 = jreshape(jperm(Ti, 1, 4, 2, 3), ov, ov)                                # :371
    scr4 = jreshape(jperm(WmBEj, 1, 3, 2, 4), ov, ov)                             # :372
    tmp = gemm("T", "N", 1.0, scr2, scr4, 0.0, None)                              # :374
    x = x + tmp                                                                   # :375
    d = jperm(jreshape(x, o, v, v, o), 1, 4, 3, 2)                                # :376
    scr1 = jreshape(jperm(d, 2, 3, 4, 1), ov, ov) + tmp                           # :379-380
    d = jperm(jreshape(scr1, o, v, v, o), 4, 1, 2, 3)                             # :381
    scr1 = jreshape(jperm(d, 2, 4, 3, 1), ov, ov)                                 # :383
    scr2 = jreshape(jperm(Ti, 1, 3, 2, 4), ov, ov)                                # :384
    scr1 = gemm("N", "N", 1.0, scr2, scr4, 1.0, scr1)                             # :385
    scr2 = 2 * scr2 - jreshape(jperm(Ti, 2, 3, 1, 4), ov, ov)                     # :387-388
    scr1 = gemm("N", "N", 1.0, scr2, scr3, 1.0, scr1)                             # :389
    return jperm(jreshape(scr1, o, v, v, o), 4, 1, 3, 2) / D                      # :391


def m_residual_update(T, oovv, vvvv, oooo, ovov, ovvo, D):
    """One mRCCD sweep without DIIS (the intermediate order of mRCCD.jl:159-166)."""
    Wabef = m_Wabef(vvvv, oovv, T)
    WmBeJ = m_WmBeJ(ovvo, oovv, T)
    WmBEj = m_WmBEj(oovv, ovov, T)
    Wmnij = m_Wmnij(oooo, oovv, T)
    Fae = m_Fae(T, oovv)
    Fmi = m_Fmi(T, oovv)
    return m_T2(T, Fae, Fmi, WmBeJ, WmBEj, Wabef, Wmnij, oovv, D)


class DIIS:
    """DIIS of mRCCD.jl:138-208, storage dtype selectable.

    ``vals`` starts with the initial amplitudes (:64) and each error pairs with
    ``vals[k+1]``; at most ``max_diis`` values are kept (:180-183), B[k,l] is
    the dot product of errors (:188-192), its error block is scaled by
    max|B| (:194), and the new amplitudes are sum_k c_k vals[k+1] (:199-202).
    The reference stores vectors and B in Float32 (:64-65,171,175,185);
    ``dtype=np.float64`` is the FP64 variant used by the GPU library.
    """

    def __init__(self, T0, max_diis=6, dtype=np.float64):
        self.dtype = dtype
        self.max_diis = max_diis
        self.vals = [np.array(T0, dtype=dtype)]
        self.errs = []

    def push_extrapolate(self, Tnew, Told):
        dt = self.dtype
        err = (Tnew - Told).ravel()
        self.vals.append(np.array(Tnew, dtype=dt))
        self.errs.append(np.array(err, dtype=dt))
        if len(self.vals) > self.max_diis:
            self.vals.pop(0)
            self.errs.pop(0)
        m = len(self.vals) - 1
        B = -np.ones((m + 1, m + 1), dtype=dt)
        B[m, m] = 0
        for k in range(m):
            for l in range(m):
                B[k, l] = np.dot(self.errs[k], self.errs[l])
        B[:m, :m] /= np.max(np.abs(B[:m, :m]))
        rhs = np.zeros(m + 1, dtype=dt)
        rhs[m] = -1
        c = np.linalg.inv(B) @ rhs
        out = np.zeros(Tnew.shape, dtype=dt)
        for k in range(m):
            out = out + dt(c[k]) * self.vals[k + 1]
        return out.astype(np.float64), float(np.linalg.norm(err))


def do_rccd(wfn, maxit=40, return_T2=False, guess="zero", diis=True, max_diis=6,
            diis_dtype=np.float64, r_conv=1e-7, e_conv=None, log=None, form="m",
            integrals=None):
    """mRCCD.do_rccd (mRCCD.jl:38-118) with the options the GPU library honours.

    guess: "zero" (mRCCD T2_init!, :239-256), "mp2" (oovv/D, mRCCSD.jl:66),
    "ovov" ((ij|ab)/D, RCCD.jl:145-160).  Convergence: stop when the
    un-extrapolated step norm < r_conv (:106,206) and, if e_conv is given,
    |dE| < e_conv.  ``form`` picks the GEMM ("m") or einsum ("jl") sweep.
    """
    o, eps = wfn.nalpha, wfn.epsa
    if integrals is None:
        integrals = make_rccd_integrals(wfn)
    oovv, ovov, ovvo, oooo, vvvv = integrals
    D = denominators(eps, o)
    if guess == "zero":
        T = np.zeros_like(oovv)
    elif guess == "mp2":
        T = oovv / D
    elif guess == "ovov":
        T = np.transpose(ovov, (0, 2, 1, 3)) / D
    else:
        raise ValueError(guess)
    sweep = m_residual_update if form == "m" else jl_cciter
    dii = DIIS(T, max_diis, diis_dtype) if diis else None
    e_old = ccenergy(T, oovv)
    niter = 0
    for i in range(maxit):
        Tn = sweep(T, oovv, vvvv, oooo, ovov, ovvo, D)
        if dii is not None:
            T_next, rms = dii.push_extrapolate(Tn, T)
        else:
            rms = float(np.linalg.norm(Tn - T))
            T_next = Tn
        T = T_next
        niter = i + 1
        e = ccenergy(T, oovv)
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
    e = ccenergy(T, oovv)
    return (e, T, niter) if return_T2 else e
