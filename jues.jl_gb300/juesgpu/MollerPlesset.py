"""Mirror of ``JuES.MollerPlesset.do_rmp2`` (src/MollerPlesset/RMP2.jl:11-45)."""
import ctypes as C
import ctypes as C_

import numpy as np

from . import _lib


def do_rmp2(refWfn, *, precision: str = "fp64", device: int = 0, doprint: bool = False,
            **kwargs) -> float:
    """Closed-shell MP2 correlation energy: get_eri(wfn,"OOVV") then the pair sum (RMP2.jl:27-41)."""
    g = _lib.f64(refWfn.ao_eri)
    Co = _lib.f64(refWfn.Cao)
    Cv = _lib.f64(refWfn.Cav)
    eps = _lib.f64(refWfn.epsa)
    e = C.c_double()
    ctx = _lib.context(device)
    _lib.check(ctx.lib.jues_rmp2(ctx.h, _lib.ptr(g), g.shape[0], _lib.ptr(Co), Co.shape[1],
                                 _lib.ptr(Cv), Cv.shape[1], _lib.ptr(eps), _lib.PREC[precision],
                                 C.byref(e), None))
    if doprint:
        print(f"   @RMP2 {e.value:>20.17f} Eh")
    return e.value


def do_df_rmp2(refWfn, pqP, Jpqh=None, *, precision: str = "fp64", device: int = 0) -> float:
    """Density-fitted MP2 (src/MollerPlesset/DF-RMP2.jl:1-46).

    ``pqP`` (n x n x naux) and ``Jpqh`` = J^-1/2 (naux x naux) are what ``setup_df``
    (src/Backend/DF.jl:30-51) returns; the reference builds them from psi4, which this
    library does not wrap.  With ``Jpqh=None``, ``pqP`` is taken as the fitted b[mu,nu,Q].
    """
    b = _lib.f64(pqP)
    if b.ndim != 3 or b.shape[0] != b.shape[1]:
        raise ValueError("pqP must be n x n x naux")
    n, _, naux = b.shape
    J = None
    if Jpqh is not None:
        J = _lib.f64(Jpqh)
        if J.shape != (naux, naux):
            raise ValueError("Jpqh must be naux x naux")
    Co = _lib.f64(refWfn.Cao)
    Cv = _lib.f64(refWfn.Cav)
    eps = _lib.f64(refWfn.epsa)
    e = C.c_double()
    ctx = _lib.context(device)
    _lib.check(ctx.lib.jues_df_rmp2(ctx.h, _lib.ptr(b), n, naux, _lib.ptr(J),
                                    _lib.ptr(Co), Co.shape[1], _lib.ptr(Cv), Cv.shape[1], _lib.ptr(eps),
                                    _lib.PREC[precision], C.byref(e)))
    return e.value


def rmp2_adjoint(refWfn=None, *, gao=None, C=None, nocc=None, eps=None, e_bar: float = 1.0,
                 want_gao: bool = True, want_C: bool = True, precision: str = "fp64", device: int = 0):
    """(E, dE/dgao * e_bar, dE/dC * e_bar) of the closed-shell MP2 energy.

    C is the full n x n MO matrix (occupied columns first).  The gradient with respect to
    the AO integrals treats every element as independent; dE/dC assumes 8-fold symmetric
    integrals.  Either pass a Wfn or gao, C, nocc, eps.
    """
    if refWfn is not None:
        gao, C, nocc, eps = refWfn.ao_eri, refWfn.Ca, refWfn.nalpha, refWfn.epsa
    g = _lib.f64(gao)
    Cm = _lib.f64(C)
    e = _lib.f64(eps)
    n = g.shape[0]
    gb = np.empty_like(g, order="F") if want_gao else None
    cb = np.empty_like(Cm, order="F") if want_C else None
    E = C_.c_double()
    ctx = _lib.context(device)
    _lib.check(ctx.lib.jues_rmp2_adjoint(ctx.h, _lib.ptr(g), n, _lib.ptr(Cm), int(nocc), _lib.ptr(e),
                                         _lib.PREC[precision], float(e_bar), C_.byref(E), _lib.ptr(gb),
                                         _lib.ptr(cb)))
    return E.value, gb, cb


def batch_rmp2(systems, *, e_bar: float = 1.0, adjoint: bool = False, precision: str = "fp64",
               device: int = 0):
    """MP2 energies (and adjoints) of many independent systems in one CUDA graph.

    systems: iterable of (gao, C, nocc, eps) or Wfn objects.  Returns (energies, gao_bars,
    C_bars, info) with the gradient lists None unless ``adjoint``.  ``precision`` "fp64" runs
    grouped FP64 GETTs; the split forms let each stage's autotuning pick the grouped
    three-plane tcgen05 GEMM where every system's contraction has K <= 64.
    """
    items = []
    for s in systems:
        if hasattr(s, "ao_eri"):
            s = (s.ao_eri, s.Ca, s.nalpha, s.epsa)
        g, Cm, o, e = s
        items.append((_lib.f64(g), _lib.f64(Cm), int(o), _lib.f64(e)))
    nsys = len(items)
    arr = (_lib.MP2System * nsys)()
    for k, (g, Cm, o, e) in enumerate(items):
        arr[k] = _lib.MP2System(g.shape[0], o, _lib.ptr(g), _lib.ptr(Cm), _lib.ptr(e))
    energies = np.zeros(nsys)
    gbs = cbs = None
    gptr = cptr = None
    if adjoint:
        gbs = [np.empty_like(g, order="F") for g, _, _, _ in items]
        cbs = [np.empty_like(Cm, order="F") for _, Cm, _, _ in items]
        gptr = (_lib.DP * nsys)(*[_lib.ptr(x) for x in gbs])
        cptr = (_lib.DP * nsys)(*[_lib.ptr(x) for x in cbs])
    info = _lib.BatchInfo()
    ctx = _lib.context(device)
    _lib.check(ctx.lib.jues_batch_rmp2(ctx.h, nsys, arr, _lib.PREC[precision], float(e_bar), _lib.ptr(energies),
                                       gptr, cptr, C_.byref(info)))
    return energies, gbs, cbs, info
