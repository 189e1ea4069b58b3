"""Mirror of ``JuES.IntegralTransformation.get_eri`` (src/Backend/IntegralTransformation.jl:38-101)."""
import numpy as np

from . import _lib


def block_shape(wfn, eri_string: str, notation: str = "phys", fcn: int = 0):
    s = eri_string
    if notation == "phys":
        s = s[0] + s[2] + s[1] + s[3]
    dims = []
    for ch in s:
        if ch in "oO":
            dims.append(wfn.nalpha - fcn)
        elif ch in "vV":
            dims.append(wfn.nvira)
        else:
            raise ValueError(f"Invalid string given to get_eri: {eri_string}")
    if notation == "phys":
        dims = [dims[0], dims[2], dims[1], dims[3]]
    return tuple(dims)


def get_eri(wfn, eri_string: str, notation: str = "phys", fcn: int = 0, *,
            precision: str = "fp64", device: int = 0) -> np.ndarray:
    """MO integral block for a closed-shell ``Wfn``; ``notation`` is "phys" or "chem"."""
    if len(eri_string.encode()) != 4:
        raise ValueError(f"Invalid string given to get_eri: {eri_string}")
    shape = block_shape(wfn, eri_string, notation, fcn)
    g = _lib.f64(wfn.ao_eri)
    Co = _lib.f64(wfn.Cao)
    Cv = _lib.f64(wfn.Cav)
    n = g.shape[0]
    out = np.empty(shape, dtype=np.float64, order="F")
    ctx = _lib.context(device)
    _lib.check(ctx.lib.jues_get_eri(ctx.h, _lib.ptr(g), n, _lib.ptr(Co), Co.shape[1], _lib.ptr(Cv),
                                    Cv.shape[1], eri_string.encode(), 1 if notation == "phys" else 0,
                                    fcn, _lib.PREC[precision], _lib.ptr(out)))
    return out


def get_fock(wfn, spin: str = "alpha", *, device: int = 0) -> np.ndarray:
    """``get_fock(wfn; spin)`` (src/Backend/IntegralTransformation.jl:119-141): the Fock matrix
    of the determinant in the basis of ``wfn.Ca`` (``Cb`` for beta), built on the device."""
    import ctypes as C
    sp = spin.lower()
    if sp in ("alpha", "up", "a"):
        Cm, Co = wfn.Ca, wfn.Cao
    elif sp in ("beta", "down", "b"):
        Cm, Co = wfn.Cb, wfn.Cbo
    else:
        raise ValueError(f"Invalid Spin option given to get_fock: {spin}")
    g = _lib.f64(wfn.ao_eri)
    h = _lib.f64(wfn.hao)
    Cm = _lib.f64(Cm)
    n, nmo = Cm.shape
    f = np.empty((nmo, nmo), order="F")
    ctx = _lib.context(device)
    _lib.check(ctx.lib.jues_get_fock(ctx.h, _lib.ptr(g), _lib.ptr(h), n, _lib.ptr(Cm), nmo,
                                     int(np.asarray(Co).shape[1]), _lib.ptr(f)))
    return f
