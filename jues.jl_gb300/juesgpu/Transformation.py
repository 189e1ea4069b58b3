"""Mirror of ``JuES.Transformation`` (src/Backend/Transformation.jl)."""
import ctypes as C

import numpy as np

from . import _lib


def tei_transform(gao, C1, C2=None, C3=None, C4=None, name: str = "default", *,
                  precision: str = "fp64", device: int = 0) -> np.ndarray:
    """(C1 C2|C3 C4)[i,a,j,b] = sum C1[mu,i] C2[nu,a] C3[lam,j] C4[sig,b] gao[mu,nu,lam,sig].

    ``tei_transform(gao, C)`` is the 2-argument form (Transformation.jl:15-20);
    ``name`` only named the disk-cache files of the reference and is ignored.
    """
    if C2 is None and C3 is None and C4 is None:
        C2 = C3 = C4 = C1
    if C2 is None or C3 is None or C4 is None:
        raise TypeError("tei_transform takes C or C1, C2, C3, C4")
    g = _lib.f64(gao)
    Cs = [_lib.f64(c) for c in (C1, C2, C3, C4)]
    n = g.shape[0]
    if g.shape != (n, n, n, n):
        raise ValueError("gao must be n^4")
    for c in Cs:
        if c.ndim != 2 or c.shape[0] != n:
            raise ValueError("each C must be nbf x d")
    d = [c.shape[1] for c in Cs]
    out = np.empty(d, dtype=np.float64, order="F")
    ctx = _lib.context(device)
    _lib.check(ctx.lib.jues_tei_transform(ctx.h, _lib.ptr(g), n,
                                          _lib.ptr(Cs[0]), d[0], _lib.ptr(Cs[1]), d[1],
                                          _lib.ptr(Cs[2]), d[2], _lib.ptr(Cs[3]), d[3],
                                          _lib.PREC[precision], _lib.ptr(out)))
    return out
