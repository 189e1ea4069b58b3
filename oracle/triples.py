"""Closed-shell (T) energy correction (oracle; test infrastructure).

Restates ``compute_pT`` (src/CoupledCluster/PerturbativeTriples.jl:35-138) with numpy:
for each occupied triple i >= j >= k, W[a,b,c] is the sum of the six permuted
(vv|vo)·T2 - (vo|oo)·T2 products (:104-111), V adds the three (vo|vo)·T1 terms (:113),
and the energy sums over a >= b >= c with the reference's weights (:117-131).

Inputs are chemists' notation, column-major in the reference: ``Vvvvo[a,b,c,i] = (ab|ci)``,
``Vvooo[a,i,j,k] = (ai|jk)``, ``Vvovo[a,i,b,j] = (ai|bj)``; ``fo``/``fv`` are the Fock
diagonals.  ``integrals_from_cc`` builds them from the physicists' blocks the CC code uses,
the same way AutoRCCSD.jl:295-297 permutes get_eri's OVVV, OOOV and OOVV.
"""
import numpy as np


def integrals_from_cc(ovvv, ooov, oovv):
    """AutoRCCSD.jl:295-297: Vvvvo = permutedims(OVVV,[4,2,3,1]), Vvooo = permutedims(OOOV,
    [4,2,1,3]), Vvovo = permutedims(OOVV,[3,1,4,2]) (Julia permutedims: out dim d = in dim p[d])."""
    Vvvvo = np.transpose(ovvv, (3, 1, 2, 0))
    Vvooo = np.transpose(ooov, (3, 1, 0, 2))
    Vvovo = np.transpose(oovv, (2, 0, 3, 1))
    return Vvvvo, Vvooo, Vvovo


def _w_ijk(i, j, k, T2, Vvvvo, Vvooo):
    """PerturbativeTriples.jl:104-111."""
    E = np.einsum
    W = (E("bda,cd->abc", Vvvvo[:, :, :, i], T2[k, j]) - E("cl,lab->abc", Vvooo[:, k, j, :], T2[i])
         + E("cda,bd->abc", Vvvvo[:, :, :, i], T2[j, k]) - E("bl,lac->abc", Vvooo[:, j, k, :], T2[i])
         + E("adc,bd->abc", Vvvvo[:, :, :, k], T2[j, i]) - E("bl,lca->abc", Vvooo[:, j, i, :], T2[k])
         + E("bdc,ad->abc", Vvvvo[:, :, :, k], T2[i, j]) - E("al,lcb->abc", Vvooo[:, i, j, :], T2[k])
         + E("cdb,ad->abc", Vvvvo[:, :, :, j], T2[i, k]) - E("al,lbc->abc", Vvooo[:, i, k, :], T2[j])
         + E("adb,cd->abc", Vvvvo[:, :, :, j], T2[k, i]) - E("cl,lba->abc", Vvooo[:, k, i, :], T2[j]))
    return W


def compute_pT(T1, T2, Vvvvo, Vvooo, Vvovo, fo, fv):
    """compute_pT (PerturbativeTriples.jl:35-138); returns E(T)."""
    o, v = T1.shape
    a_, b_, c_ = np.meshgrid(np.arange(v), np.arange(v), np.arange(v), indexing="ij")
    keep = (a_ >= b_) & (b_ >= c_)
    a_, b_, c_ = a_[keep], b_[keep], c_[keep]
    dab = (a_ == b_).astype(float)
    dbc = (b_ == c_).astype(float)
    Et = 0.0
    for i in range(o):
        for j in range(i + 1):
            for k in range(j + 1):
                W = _w_ijk(i, j, k, T2, Vvvvo, Vvooo)
                V = (W + Vvovo[:, j, :, k][None, :, :] * T1[i][:, None, None]
                     + Vvovo[:, i, :, k][:, None, :] * T1[j][None, :, None]
                     + Vvovo[:, i, :, j][:, :, None] * T1[k][None, None, :])
                w = lambda p, q, r: W[p, q, r]     # noqa: E731
                vv = lambda p, q, r: V[p, q, r]    # noqa: E731
                X = (w(a_, b_, c_) * vv(a_, b_, c_) + w(a_, c_, b_) * vv(a_, c_, b_)
                     + w(b_, a_, c_) * vv(b_, a_, c_) + w(b_, c_, a_) * vv(b_, c_, a_)
                     + w(c_, a_, b_) * vv(c_, a_, b_) + w(c_, b_, a_) * vv(c_, b_, a_))
                Y = vv(a_, b_, c_) + vv(b_, c_, a_) + vv(c_, a_, b_)
                Z = vv(a_, c_, b_) + vv(b_, a_, c_) + vv(c_, b_, a_)
                En = ((Y - 2 * Z) * (w(a_, b_, c_) + w(b_, c_, a_) + w(c_, a_, b_))
                      + (Z - 2 * Y) * (w(a_, c_, b_) + w(b_, a_, c_) + w(c_, b_, a_)) + 3 * X)
                Dd = fo[i] + fo[j] + fo[k] - fv[a_] - fv[b_] - fv[c_]
                dij = float(i == j)
                djk = float(j == k)
                Et += float(np.sum(En * (2 - dij - djk) / (Dd * (1 + dab + dbc))))
    return Et


def compute_pT_loops(T1, T2, Vvvvo, Vvooo, Vvovo, fo, fv):
    """The same with the reference's scalar energy loop (:117-131); small cases only."""
    o, v = T1.shape
    Et = 0.0
    for i in range(o):
        for j in range(i + 1):
            for k in range(j + 1):
                W = _w_ijk(i, j, k, T2, Vvvvo, Vvooo)
                V = (W + np.einsum("bc,a->abc", Vvovo[:, j, :, k], T1[i])
                     + np.einsum("ac,b->abc", Vvovo[:, i, :, k], T1[j])
                     + np.einsum("ab,c->abc", Vvovo[:, i, :, j], T1[k]))
                for a in range(v):
                    for b in range(a + 1):
                        for c in range(b + 1):
                            Dd = fo[i] + fo[j] + fo[k] - fv[a] - fv[b] - fv[c]
                            X = (W[a, b, c] * V[a, b, c] + W[a, c, b] * V[a, c, b] + W[b, a, c] * V[b, a, c]
                                 + W[b, c, a] * V[b, c, a] + W[c, a, b] * V[c, a, b] + W[c, b, a] * V[c, b, a])
                            Y = V[a, b, c] + V[b, c, a] + V[c, a, b]
                            Z = V[a, c, b] + V[b, a, c] + V[c, b, a]
                            En = ((Y - 2 * Z) * (W[a, b, c] + W[b, c, a] + W[c, a, b])
                                  + (Z - 2 * Y) * (W[a, c, b] + W[b, a, c] + W[c, b, a]) + 3 * X)
                            Et += En * (2 - (i == j) - (j == k)) / (Dd * (1 + (a == b) + (b == c)))
    return Et
