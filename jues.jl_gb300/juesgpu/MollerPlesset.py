"""Mirror of ``JuES.MollerPlesset.do_rmp2`` (src/MollerPlesset/RMP2.jl:11-45)."""
import ctypes as C

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
