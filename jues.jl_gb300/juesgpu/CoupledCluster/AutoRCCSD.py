"""Mirror of ``JuES.CoupledCluster.AutoRCCSD`` (src/CoupledCluster/AutoRCCSD.jl:193-300).

CCSD from the Fock matrix of the given orbitals (``get_fock``), so non-canonical orbitals and
non-Hartree-Fock references work: the off-diagonal Fock blocks enter the equations and the
diagonal forms the resolvents.  Options are the CoupledCluster module defaults
(CoupledCluster.jl:36-43): ``cc_max_iter = 50``, ``cc_max_rms = 1e-10``, ``cc_e_conv = 1e-10``,
``diis = False``, ``do_pT = False``, ``fcn = 0``.  The reference prints the energies and
returns nothing; this returns the CCSD correlation energy, and ``(E, E(T))`` with ``do_pT``.
"""
import ctypes as C
import warnings

import numpy as np

from .. import _lib
from . import defaults
from ._solve import make_opts


def do_rccsd(wfn, *, precision="fp64", device=0, return_T=False, **kwargs):
    opt = dict(defaults)
    opt.update(kwargs)
    nelec = wfn.nalpha + wfn.nbeta
    if nelec % 2 != 0:
        raise ValueError(f"Number of electrons must be even for RHF. Given {nelec}")
    opts = make_opts(maxit=opt["cc_max_iter"], e_conv=opt["cc_e_conv"], r_conv=opt["cc_max_rms"],
                     diis=opt["diis"], precision=precision, guess="mp2", refine=0)
    g = _lib.f64(wfn.ao_eri)
    h = _lib.f64(wfn.hao)
    Cm = _lib.f64(wfn.Ca)
    n, nmo = Cm.shape
    ndocc = nelec // 2
    fcn = int(opt["fcn"])
    o, v = ndocc - fcn, nmo - ndocc
    t1 = np.empty((o, v), order="F")
    T2 = np.empty((o, o, v, v), order="F")
    cap = max(1, opts.maxit)
    log = (_lib.IterLog * cap)()
    e = C.c_double()
    ept = C.c_double()
    nit = C.c_int()
    ctx = _lib.context(device)
    st = ctx.lib.jues_auto_rccsd(ctx.h, _lib.ptr(g), _lib.ptr(h), n, _lib.ptr(Cm), nmo, ndocc, fcn, C.byref(opts),
                                 1 if opt["do_pT"] else 0, C.byref(e), C.byref(ept), _lib.ptr(t1), _lib.ptr(T2),
                                 log, cap, C.byref(nit))
    if st == _lib.ENOTCONV:
        warnings.warn(_lib.last_error(), RuntimeWarning, stacklevel=2)
    else:
        _lib.check(st)
    out = (e.value, ept.value) if opt["do_pT"] else e.value
    if return_T:
        recs = [(r.iter, r.energy, r.rnorm, r.ms, r.precision) for r in log[: nit.value]]
        return out, t1, T2, recs
    return out
