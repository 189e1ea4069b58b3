"""Density-fitted closed-shell CCD (oracle; test infrastructure).

Restates ``src/CoupledCluster/DF-RCCD.jl`` term by term on the MO factors of the fitted
three-index tensor b[mu,nu,Q] (``DF.make_bmunu``, src/Backend/DF.jl:52-57).  The reference
iterates exactly ``maxit`` Jacobi sweeps from T2 = (ia|jb)/D with no DIIS and no convergence
test (DF-RCCD.jl:11-54).

``variant="reference"`` keeps DF-RCCD.jl's WmBeJ, whose last term contracts
bov[m,e,Q] bov[n,f,Q] = (me|nf) with T[n,j,f,b] (:247-253); RCCD.jl:400 reads that term as
<nm|ef> = (ne|mf).  ``variant="rccd"`` uses RCCD.jl's order, which makes the iteration
RCCD's on the fitted integrals.
"""
import numpy as np


def E(*a):
    return np.einsum(*a, optimize=True)


def make_df_rccd_integrals(wfn, b):
    """DF-RCCD.jl:78-89: bov, bvo, boo, bvv from b[mu,nu,Q]."""
    Co, Cv = wfn.Cao, wfn.Cav
    bov = E("mi,mnQ,na->iaQ", Co, b, Cv)
    bvo = E("ma,mnQ,ni->aiQ", Cv, b, Co)
    boo = E("mi,mnQ,nj->ijQ", Co, b, Co)
    bvv = E("ma,mnQ,nb->abQ", Cv, b, Cv)
    return bov, bvo, boo, bvv


def denominators(eps, o):
    """form_Dijab (src/CoupledCluster/Denominators.jl:14-33)."""
    eo, ev = eps[:o], eps[o:]
    return eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None] - ev[None, None, None, :]


def ccenergy(T, bov):
    """DF-RCCD.jl:90-111: sum (ia|jb) (2 T[i,j,a,b] - T[j,i,a,b])."""
    bAB = E("iaQ,jbQ->ijab", bov, bov)
    return float(np.sum(bAB * (2.0 * T - np.transpose(T, (1, 0, 2, 3)))))


def T2_init(bov, D):
    """DF-RCCD.jl:112-137: T[i,j,a,b] = (ia|jb) / D."""
    return E("iaQ,jbQ->ijab", bov, bov) / D


def form_Fae(T, bov):
    """DF-RCCD.jl:144-153."""
    return -E("meQ,nfQ,mnaf->ae", bov, bov, 2.0 * T - np.transpose(T, (1, 0, 2, 3)))


def form_Fmi(T, bov):
    """DF-RCCD.jl:162-171."""
    return E("meQ,nfQ,inef->mi", bov, bov, 2.0 * T - np.transpose(T, (0, 1, 3, 2)))


def form_Wmnij(boo, bov, T):
    """DF-RCCD.jl:230-238."""
    return E("miQ,njQ->mnij", boo, boo) + E("ijef,meQ,nfQ->mnij", T, bov, bov) / 2.0


def form_WmBeJ(bov, bvo, T, variant="reference"):
    """DF-RCCD.jl:247-253 (``variant="rccd"``: the last term as RCCD.jl:400)."""
    mnef = E("meQ,nfQ->mnef", bov, bov)
    W = E("meQ,bjQ->mbej", bov, bvo)
    W += E("mnef,njfb->mbej", mnef, 2.0 * T - np.transpose(T, (1, 0, 2, 3))) / 2.0
    if variant == "reference":
        W -= E("mnef,njfb->mbej", mnef, T) / 2.0
    else:
        W -= E("nmef,njfb->mbej", mnef, T) / 2.0
    return W


def form_WmBEj(boo, bvv, bov, T):
    """DF-RCCD.jl:262-270."""
    return -E("mjQ,beQ->mbej", boo, bvv) + E("jnfb,neQ,mfQ->mbej", T, bov, bov) / 2.0


def form_T2(T, Fae, Fmi, WmBeJ, WmBEj, Wmnij, bov, bvv, D):
    """DF-RCCD.jl:172-221."""
    mnef = E("meQ,nfQ->mnef", bov, bov)
    R = E("iaQ,jbQ->ijab", bov, bov)
    R += E("ijae,be->ijab", T, Fae) + E("jibe,ae->ijab", T, Fae)
    R -= E("imab,mj->ijab", T, Fmi) + E("mjab,mi->ijab", T, Fmi)
    R += E("mnab,mnij->ijab", T, Wmnij)
    R += E("ijmn,mnab->ijab", E("ijef,mnef->ijmn", T, mnef), T) / 2.0
    R += E("ijef,abef->ijab", T, E("aeQ,bfQ->abef", bvv, bvv))     # (ae|bf), contracted over Q first
    R += E("imae,mbej->ijab", T, WmBeJ) * 2.0
    R -= E("miae,mbej->ijab", T, WmBeJ)
    R += E("imae,mbej->ijab", T, WmBEj)
    R += E("mibe,maej->ijab", T, WmBEj)
    R += E("mjae,mbei->ijab", T, WmBEj)
    R += E("jmbe,maei->ijab", T, WmBeJ) * 2.0
    R -= E("mjbe,maei->ijab", T, WmBeJ)
    R += E("jmbe,maei->ijab", T, WmBEj)
    return R / D


def do_df_rccd(wfn, b, maxit=40, variant="reference", return_T2=False, log=None):
    """DF-RCCD.jl:11-54.  ``log`` (a list) receives (iteration, energy) after each sweep."""
    o = wfn.nalpha
    bov, bvo, boo, bvv = make_df_rccd_integrals(wfn, b)
    D = denominators(wfn.epsa, o)
    T = T2_init(bov, D)
    for it in range(maxit):
        WmBeJ = form_WmBeJ(bov, bvo, T, variant)
        WmBEj = form_WmBEj(boo, bvv, bov, T)
        Wmnij = form_Wmnij(boo, bov, T)
        Fae = form_Fae(T, bov)
        Fmi = form_Fmi(T, bov)
        T = form_T2(T, Fae, Fmi, WmBeJ, WmBEj, Wmnij, bov, bvv, D)
        if log is not None:
            log.append((it + 1, ccenergy(T, bov)))
    e = ccenergy(T, bov)
    return (e, T) if return_T2 else e
