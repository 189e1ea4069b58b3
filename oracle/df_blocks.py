"""MO integral blocks of a B-factored synthetic system (oracle; test infrastructure).

For (mu nu|lam sig) = sum_P B[P,mu,nu] B[P,lam,sig] the MO blocks follow from the
half-transformed factors B[P,p,q] = C^T B[P] C at O(naux n^3) instead of the O(n^5) four-index
transform; the blocks are the same numbers (up to rounding) as get_eri's.  Used to prepare CPU
baseline timings of the CC sweep at sizes where the n^4 transform would dominate.
"""
import numpy as np


def rccd_blocks_from_B(B, C, o):
    naux, n, _ = B.shape
    Co, Cv = C[:, :o], C[:, o:]
    Boo = np.einsum("Pmn,mi,nj->Pij", B, Co, Co, optimize=True)
    Bov = np.einsum("Pmn,mi,na->Pia", B, Co, Cv, optimize=True)
    Bvv = np.einsum("Pmn,ma,nb->Pab", B, Cv, Cv, optimize=True)
    v = n - o

    def chem(X, Y):
        a, b = X.shape[1:]
        c, d = Y.shape[1:]
        return (X.reshape(naux, a * b).T @ Y.reshape(naux, c * d)).reshape(a, b, c, d)

    oovv = np.ascontiguousarray(chem(Bov, Bov).transpose(0, 2, 1, 3))     # <ij|ab> = (ia|jb)
    ovov = np.ascontiguousarray(chem(Boo, Bvv).transpose(0, 2, 1, 3))     # <ia|jb> = (ij|ab)
    ovvo = np.ascontiguousarray(chem(Bov, Bov.transpose(0, 2, 1)).transpose(0, 2, 1, 3))
    oooo = np.ascontiguousarray(chem(Boo, Boo).transpose(0, 2, 1, 3))
    vvvv = np.ascontiguousarray(chem(Bvv, Bvv).transpose(0, 2, 1, 3))
    return oovv, ovov, ovvo, oooo, vvvv
