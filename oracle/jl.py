"""Julia array semantics in numpy (test infrastructure; see package header).

``jperm(X, p...)``  == Julia ``permutedims(X, (p...))`` with 1-based ``p``.
``jreshape(X, d...)`` == Julia ``reshape(X, d...)`` (column-major).
``gemm(tA, tB, alpha, A, B, beta, C)`` == ``BLAS.gemm!`` returning the new C.
"""
import numpy as np


def jperm(X, *p):
    return np.transpose(X, [q - 1 for q in p])


def jreshape(X, *dims):
    return np.reshape(X, dims, order="F")


def gemm(tA, tB, alpha, A, B, beta, C):
    a = A.T if tA == "T" else A
    b = B.T if tB == "T" else B
    out = alpha * (a @ b)
    if beta != 0.0:
        out = out + beta * C
    return out
