"""Mirror of ``JuES.CoupledCluster.PerturbativeTriples`` (src/CoupledCluster/PerturbativeTriples.jl).

``compute_pT`` takes the reference's keyword arguments: chemists'-notation integrals
``Vvvvo[a,b,c,i] = (ab|ci)``, ``Vvooo[a,i,j,k] = (ai|jk)``, ``Vvovo[a,i,b,j] = (ai|bj)``, the
CCSD amplitudes and the Fock diagonals.  A CCSD session computes the same from its resident
blocks with ``CCSession.pT()``.
"""
import ctypes as C

from .. import _lib


def compute_pT(*, T1, T2, Vvvvo, Vvooo, Vvovo, fo, fv, precision="fp64", device=0):
    t1 = _lib.f64(T1)
    o, v = t1.shape
    t2 = _lib.f64(T2)
    arrs = {"T2": (t2, (o, o, v, v)), "Vvvvo": (_lib.f64(Vvvvo), (v, v, v, o)),
            "Vvooo": (_lib.f64(Vvooo), (v, o, o, o)), "Vvovo": (_lib.f64(Vvovo), (v, o, v, o)),
            "fo": (_lib.f64(fo), (o,)), "fv": (_lib.f64(fv), (v,))}
    for name, (a, shape) in arrs.items():
        if a.shape != shape:
            raise ValueError(f"{name} must have shape {shape}, got {a.shape}")
    e = C.c_double()
    ctx = _lib.context(device)
    _lib.check(ctx.lib.jues_pT(ctx.h, _lib.ptr(t1), _lib.ptr(t2), _lib.ptr(arrs["Vvvvo"][0]),
                               _lib.ptr(arrs["Vvooo"][0]), _lib.ptr(arrs["Vvovo"][0]), _lib.ptr(arrs["fo"][0]),
                               _lib.ptr(arrs["fv"][0]), o, v, _lib.PREC[precision], C.byref(e)))
    return e.value
