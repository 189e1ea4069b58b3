"""Closed-shell MP2 (oracle; test infrastructure).

Follows ``src/MollerPlesset/RMP2.jl:11-45``: ``moeri = get_eri(wfn,"OOVV")`` (:24)
then E = sum_{ijab} K[i,j,a,b](2K[i,j,a,b] - K[i,j,b,a]) /
(eps_i + eps_j - eps_{o+a} - eps_{o+b}) (:27-41).
"""
import numpy as np

from .transform import get_eri


def denominators(eps, o):
    """D[i,j,a,b] of ``form_Dijab`` (src/CoupledCluster/Denominators.jl:14-33)."""
    eo = eps[:o]
    ev = eps[o:]
    return (eo[:, None, None, None] + eo[None, :, None, None]
            - ev[None, None, :, None] - ev[None, None, None, :])


def rmp2_energy(K, eps, o):
    D = denominators(eps, o)
    return float(np.sum(K * (2.0 * K - np.transpose(K, (0, 1, 3, 2))) / D))


def rmp2_energy_loops(K, eps, o):
    """Scalar loop exactly as RMP2.jl:27-41 (b, a, j, i order); small cases only."""
    nv = K.shape[2]
    e = 0.0
    for b in range(nv):
        for a in range(nv):
            for j in range(o):
                for i in range(o):
                    e += (K[i, j, a, b] * (2 * K[i, j, a, b] - K[i, j, b, a])
                          / (eps[i] + eps[j] - eps[o + a] - eps[o + b]))
    return e


def do_rmp2(wfn):
    K = get_eri(wfn, "OOVV")
    return rmp2_energy(K, wfn.epsa, wfn.nalpha)


def df_rmp2(wfn, pqP, Jpqh=None):
    """``do_df_rmp2`` (src/MollerPlesset/DF-RMP2.jl:1-46): b = pqP.Jpqh (:14-16; skipped
    when Jpqh is None), B_iaQ = Co^T b Cv (:17-22), then per (i, j) the (ia|jb) block and
    the same pair sum as RMP2 (:23-45)."""
    o = wfn.nalpha
    b = pqP if Jpqh is None else np.einsum("pqP,PQ->pqQ", pqP, Jpqh, optimize=True)
    Bia = np.einsum("mi,mnQ,na->iaQ", wfn.Cao, b, wfn.Cav, optimize=True)
    eps = wfn.epsa
    e = 0.0
    for i in range(o):
        for j in range(o):
            bAB = Bia[i] @ Bia[j].T                  # (ia|jb) over a, b
            D = eps[i] + eps[j] - eps[o:, None] - eps[None, o:]
            e += float(np.sum(bAB * (2.0 * bAB - bAB.T) / D))
    return e
