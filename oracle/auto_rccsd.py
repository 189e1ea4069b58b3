"""Closed-shell CCSD from a general (non-canonical) Fock matrix (oracle; test infrastructure).

Restates ``src/CoupledCluster/AutoRCCSD.jl`` term by term: ``update_energy`` (:40-51),
``update_amp`` (:67-178) and the ``do_rccsd`` driver (:193-300), with ``get_fock``
(src/Backend/IntegralTransformation.jl:119-141).  The driver takes the Fock matrix of the
given orbitals, keeps its diagonal for the resolvents and its off-diagonal part in the
equations, starts from T1 = f_ov/d and T2 = <ij|ab>/D, and iterates until |dE| and the
per-element rms (||dT||/length(T), the larger of T1's and T2's) are both below their
thresholds.  ``fcn`` frozen core orbitals are dropped from the occupied range.
"""
import numpy as np

from .transform import get_eri


def E(*a):
    return np.einsum(*a, optimize=True)


def get_fock(C, Co, gao, hao):
    """IntegralTransformation.jl:119-141: f = C^T h C + 2 (pq|kk) - (pk|qk) over occupied k."""
    D = Co @ Co.T
    J = E("mnls,ls->mn", gao, D)
    K = E("mlns,ls->mn", gao, D)
    return C.T @ (hao + 2.0 * J - K) @ C


def update_energy(T1, T2, f_ov, Voovv):
    """AutoRCCSD.jl:40-51."""
    B = -E("lc,kd->lckd", T1, T1) - np.transpose(T2, (0, 2, 1, 3)) + 2.0 * np.transpose(T2, (1, 2, 0, 3))
    e = 2.0 * E("kc,kc->", f_ov, T1)
    e += E("lckd,klcd->", B, Voovv)
    e += 2.0 * E("lc,kd,lkcd->", T1, T1, Voovv)
    return float(e)


def update_amp(T1, T2, f, V, d, D):
    """AutoRCCSD.jl:67-178; returns (newT1, newT2, r1, r2)."""
    Voooo, Vooov, Voovv, Vovov, Vovvv, Vvvvv = V
    fOO, fOV, fVV = f
    t1 = T1
    t2 = T2
    n1 = np.zeros_like(T1)
    n1 += fOV
    n1 -= E("ik,ka->ia", fOO, t1)
    n1 += E("ca,ic->ia", fVV, t1)
    n1 -= E("kc,ic,ka->ia", fOV, t1, t1)
    n1 += 2.0 * E("kc,ikac->ia", fOV, t2)
    n1 -= E("kc,kiac->ia", fOV, t2)
    n1 -= E("kc,icka->ia", t1, Vovov)
    n1 += 2.0 * E("kc,kica->ia", t1, Voovv)
    n1 -= E("kicd,kadc->ia", t2, Vovvv)
    n1 += 2.0 * E("ikcd,kadc->ia", t2, Vovvv)
    n1 += -2.0 * E("klac,klic->ia", t2, Vooov)
    n1 += E("lkac,klic->ia", t2, Vooov)
    n1 += -2.0 * E("kc,la,lkic->ia", t1, t1, Vooov)
    n1 -= E("kc,id,kadc->ia", t1, t1, Vovvv)
    n1 += 2.0 * E("kc,id,kacd->ia", t1, t1, Vovvv)
    n1 += E("kc,la,klic->ia", t1, t1, Vooov)
    n1 += -2.0 * E("kc,ilad,lkcd->ia", t1, t2, Voovv)
    n1 += -2.0 * E("kc,liad,klcd->ia", t1, t2, Voovv)
    n1 += E("kc,liad,lkcd->ia", t1, t2, Voovv)
    n1 += -2.0 * E("ic,lkad,lkcd->ia", t1, t2, Voovv)
    n1 += E("ic,lkad,klcd->ia", t1, t2, Voovv)
    n1 += -2.0 * E("la,ikdc,klcd->ia", t1, t2, Voovv)
    n1 += E("la,ikcd,klcd->ia", t1, t2, Voovv)
    n1 += E("kc,id,la,lkcd->ia", t1, t1, t1, Voovv)
    n1 += -2.0 * E("kc,id,la,klcd->ia", t1, t1, t1, Voovv)
    n1 += 4.0 * E("kc,ilad,klcd->ia", t1, t2, Voovv)

    n2 = Voovv.copy()
    n2 += E("ic,jd,cdab->ijab", t1, t1, Vvvvv)
    n2 += E("ijcd,cdab->ijab", t2, Vvvvv)
    n2 += E("ka,lb,ijkl->ijab", t1, t1, Voooo)
    n2 += E("klab,ijkl->ijab", t2, Voooo)
    n2 -= E("ic,jd,ka,kbcd->ijab", t1, t1, t1, Vovvv)
    n2 -= E("ic,jd,kb,kadc->ijab", t1, t1, t1, Vovvv)
    n2 += E("ic,ka,lb,lkjc->ijab", t1, t1, t1, Vooov)
    n2 += E("jc,ka,lb,klic->ijab", t1, t1, t1, Vooov)
    n2 += E("klac,ijdb,klcd->ijab", t2, t2, Voovv)
    n2 += -2.0 * E("ikac,ljbd,klcd->ijab", t2, t2, Voovv)
    n2 += -2.0 * E("lkac,ijdb,klcd->ijab", t2, t2, Voovv)
    n2 += E("kiac,ljdb,lkcd->ijab", t2, t2, Voovv)
    n2 += E("ikac,ljbd,lkcd->ijab", t2, t2, Voovv)
    n2 += -2.0 * E("ikac,jlbd,lkcd->ijab", t2, t2, Voovv)
    n2 += E("kiac,ljbd,klcd->ijab", t2, t2, Voovv)
    n2 += -2.0 * E("kiac,jlbd,klcd->ijab", t2, t2, Voovv)
    n2 += E("ijac,lkbd,klcd->ijab", t2, t2, Voovv)
    n2 += -2.0 * E("ijac,klbd,klcd->ijab", t2, t2, Voovv)
    n2 += E("kjac,ildb,lkcd->ijab", t2, t2, Voovv)
    n2 += 4.0 * E("ikac,jlbd,klcd->ijab", t2, t2, Voovv)
    n2 += E("ijdc,lkab,klcd->ijab", t2, t2, Voovv)
    n2 += E("ic,jd,ka,lb,klcd->ijab", t1, t1, t1, t1, Voovv)
    n2 += E("ic,jd,lkab,lkcd->ijab", t1, t1, t2, Voovv)
    n2 += E("ka,lb,ijdc,lkcd->ijab", t1, t1, t2, Voovv)

    P = -E("ik,kjab->ijab", fOO, t2)
    P += E("ca,ijcb->ijab", fVV, t2)
    P += -E("kb,jika->ijab", t1, Vooov)
    P += E("jc,icab->ijab", t1, Vovvv)
    P += -E("kc,ic,kjab->ijab", fOV, t1, t2)
    P += -E("kc,ka,ijcb->ijab", fOV, t1, t2)
    P += -E("kiac,kjcb->ijab", t2, Voovv)
    P += -E("ic,ka,kjcb->ijab", t1, t1, Voovv)
    P += -E("ic,kb,jcka->ijab", t1, t1, Vovov)
    P += 2.0 * E("ikac,kjcb->ijab", t2, Voovv)
    P += -E("ikac,jckb->ijab", t2, Vovov)
    P += -E("kjac,ickb->ijab", t2, Vovov)
    P += -2.0 * E("lb,ikac,lkjc->ijab", t1, t2, Vooov)
    P += E("lb,kiac,lkjc->ijab", t1, t2, Vooov)
    P += -E("jc,ikdb,kacd->ijab", t1, t2, Vovvv)
    P += -E("jc,kiad,kbdc->ijab", t1, t2, Vovvv)
    P += -E("jc,ikad,kbcd->ijab", t1, t2, Vovvv)
    P += E("jc,lkab,lkic->ijab", t1, t2, Vooov)
    P += E("lb,ikac,kljc->ijab", t1, t2, Vooov)
    P += -E("ka,ijdc,kbdc->ijab", t1, t2, Vovvv)
    P += E("ka,ilcb,lkjc->ijab", t1, t2, Vooov)
    P += 2.0 * E("jc,ikad,kbdc->ijab", t1, t2, Vovvv)
    P += -E("kc,ijad,kbdc->ijab", t1, t2, Vovvv)
    P += 2.0 * E("kc,ijad,kbcd->ijab", t1, t2, Vovvv)
    P += E("kc,ilab,kljc->ijab", t1, t2, Vooov)
    P += -2.0 * E("kc,ilab,lkjc->ijab", t1, t2, Vooov)
    P += E("jkcd,ilab,klcd->ijab", t2, t2, Voovv)
    P += -2.0 * E("kc,jd,ilab,klcd->ijab", t1, t1, t2, Voovv)
    P += E("kc,jd,ilab,lkcd->ijab", t1, t1, t2, Voovv)
    P += -2.0 * E("kc,la,ijdb,klcd->ijab", t1, t1, t2, Voovv)
    P += E("kc,la,ijdb,lkcd->ijab", t1, t1, t2, Voovv)
    P += E("ic,ka,ljbd,klcd->ijab", t1, t1, t2, Voovv)
    P += -2.0 * E("ic,ka,jlbd,klcd->ijab", t1, t1, t2, Voovv)
    P += E("ic,ka,ljdb,lkcd->ijab", t1, t1, t2, Voovv)
    P += E("ic,lb,kjad,klcd->ijab", t1, t1, t2, Voovv)
    P += -2.0 * E("ikdc,ljab,klcd->ijab", t2, t2, Voovv)
    n2 += P + np.transpose(P, (1, 0, 3, 2))

    n1 = n1 / d
    n2 = n2 / D
    r1 = float(np.sqrt(np.sum((n1 - T1) ** 2)) / T1.size)
    r2 = float(np.sqrt(np.sum((n2 - T2) ** 2)) / T2.size)
    return n1, n2, r1, r2


def do_rccsd(wfn, cc_max_iter=50, cc_max_rms=1e-10, cc_e_conv=1e-10, fcn=0, log=None, return_T=False):
    """AutoRCCSD.do_rccsd (:193-300) without the (T) branch; returns the CCSD correlation
    energy (the reference prints it and returns nothing)."""
    ndocc = wfn.nalpha
    nmo = wfn.Ca.shape[1]
    C = wfn.Ca
    f = get_fock(C, wfn.Cao, wfn.ao_eri, wfn.hao)
    o = slice(fcn, ndocc)
    v = slice(ndocc, nmo)
    fo_d = np.diag(f)[o]
    fv_d = np.diag(f)[v]
    f = f - np.diag(np.diag(f))
    fs = (f[o, o], f[o, v], f[v, v])
    V = tuple(get_eri(wfn, s, fcn=fcn) for s in ("OOOO", "OOOV", "OOVV", "OVOV", "OVVV", "VVVV"))
    d = fo_d[:, None] - fv_d[None, :]
    D = fo_d[:, None, None, None] + fo_d[None, :, None, None] - fv_d[None, None, :, None] - fv_d[None, None, None, :]
    T1 = fs[1] / d
    T2 = V[2] / D
    Ecc = update_energy(T1, T2, fs[1], V[2])
    dE, rms, ite = 1.0, 1.0, 1
    while abs(dE) > cc_e_conv or rms > cc_max_rms:
        if ite > cc_max_iter:
            break
        T1, T2, r1, r2 = update_amp(T1, T2, fs, V, d, D)
        rms = max(r1, r2)
        old = Ecc
        Ecc = update_energy(T1, T2, fs[1], V[2])
        dE = Ecc - old
        if log is not None:
            log.append((ite, Ecc, rms))
        ite += 1
    if return_T:
        return Ecc, T1, T2, (fo_d, fv_d), V
    return Ecc
