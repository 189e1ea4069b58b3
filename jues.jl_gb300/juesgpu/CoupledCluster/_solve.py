"""Shared driver of the CC mirrors: options -> jues_cc_opts, whole solves and sessions."""
import ctypes as C
import warnings

import numpy as np

from .. import _lib


def make_opts(maxit=40, e_conv=0.0, r_conv=1e-7, diis=True, diis_size=6, precision="fp64",
              guess="zero", refine=2, transform_precision=None, ccsd_fae="rccsd") -> _lib.CCOpts:
    o = _lib.default_opts()
    o.maxit = int(maxit)
    o.e_conv = float(e_conv or 0.0)
    o.r_conv = float(r_conv or 0.0)
    o.diis = 1 if diis else 0
    o.diis_size = int(diis_size)
    o.precision = _lib.PREC[precision]
    o.guess = _lib.GUESS[guess]
    o.refine = int(refine)
    o.transform_precision = -1 if transform_precision is None else _lib.PREC[transform_precision]
    o.ccsd_fae = _lib.CCSD_FAE[ccsd_fae]
    return o


def solve(method, wfn, device=0, return_log=False, **kw):
    """method 0 = CCD, 1 = CCSD.  Returns (E, t1, T2, niter, log)."""
    opts = make_opts(**kw)
    g = _lib.f64(wfn.ao_eri)
    Co = _lib.f64(wfn.Cao)
    Cv = _lib.f64(wfn.Cav)
    eps = _lib.f64(wfn.epsa)
    n, o, v = g.shape[0], Co.shape[1], Cv.shape[1]
    T2 = np.empty((o, o, v, v), order="F")
    t1 = np.empty((o, v), order="F") if method == 1 else None
    cap = max(1, opts.maxit)
    log = (_lib.IterLog * cap)()
    e = C.c_double()
    nit = C.c_int()
    ctx = _lib.context(device)
    if method == 0:
        st = ctx.lib.jues_rccd(ctx.h, _lib.ptr(g), n, _lib.ptr(Co), o, _lib.ptr(Cv), v, _lib.ptr(eps),
                               C.byref(opts), C.byref(e), _lib.ptr(T2), log, cap, C.byref(nit))
    else:
        st = ctx.lib.jues_rccsd(ctx.h, _lib.ptr(g), n, _lib.ptr(Co), o, _lib.ptr(Cv), v,
                                _lib.ptr(eps), C.byref(opts), C.byref(e), _lib.ptr(t1), _lib.ptr(T2),
                                log, cap, C.byref(nit))
    if st == _lib.ENOTCONV:
        # the reference stops silently at maxit (mRCCD.jl:68-109); keep its behaviour
        warnings.warn(_lib.last_error(), RuntimeWarning, stacklevel=3)
    else:
        _lib.check(st)
    recs = [(r.iter, r.energy, r.rnorm, r.ms, r.precision) for r in log[: nit.value]]
    return e.value, t1, T2, nit.value, recs


def df_arrays(pqP, Jpqh):
    b = _lib.f64(pqP)
    if b.ndim != 3 or b.shape[0] != b.shape[1]:
        raise ValueError("pqP must be n x n x naux")
    J = None
    if Jpqh is not None:
        J = _lib.f64(Jpqh)
        if J.shape != (b.shape[2], b.shape[2]):
            raise ValueError("Jpqh must be naux x naux")
    return b, J


def solve_df(wfn, pqP, Jpqh=None, variant="reference", device=0, **kw):
    """CCD on density-fitted integrals (jues_df_rccd).  Returns (E, T2, niter, log)."""
    opts = make_opts(**kw)
    b, J = df_arrays(pqP, Jpqh)
    Co = _lib.f64(wfn.Cao)
    Cv = _lib.f64(wfn.Cav)
    eps = _lib.f64(wfn.epsa)
    n, naux = b.shape[0], b.shape[2]
    o, v = Co.shape[1], Cv.shape[1]
    T2 = np.empty((o, o, v, v), order="F")
    cap = max(1, opts.maxit)
    log = (_lib.IterLog * cap)()
    e = C.c_double()
    nit = C.c_int()
    ctx = _lib.context(device)
    st = ctx.lib.jues_df_rccd(ctx.h, _lib.ptr(b), n, naux, _lib.ptr(J), _lib.ptr(Co), o, _lib.ptr(Cv), v,
                              _lib.ptr(eps), C.byref(opts), _lib.DF_VARIANT[variant], C.byref(e), _lib.ptr(T2),
                              log, cap, C.byref(nit))
    if st == _lib.ENOTCONV:
        warnings.warn(_lib.last_error(), RuntimeWarning, stacklevel=3)
    else:
        _lib.check(st)
    recs = [(r.iter, r.energy, r.rnorm, r.ms, r.precision) for r in log[: nit.value]]
    return e.value, T2, nit.value, recs


class CCSession:
    """Device-resident CC problem (jues_cc_create / jues_cc_iterate)."""

    def __init__(self, method, wfn=None, *, gao=None, gao_dev_ptr=None, Cocc=None, Cvir=None,
                 eps=None, device=0, pqP=None, Jpqh=None, df_variant="reference", **kw):
        self.ctx = _lib.context(device)
        self.opts = make_opts(**kw)
        if wfn is not None:
            gao, Cocc, Cvir, eps = wfn.ao_eri, wfn.Cao, wfn.Cav, wfn.epsa
        Co, Cv, e = _lib.f64(Cocc), _lib.f64(Cvir), _lib.f64(eps)
        n = Co.shape[0]
        self.o, self.v = Co.shape[1], Cv.shape[1]
        h = _lib.VP()
        self.method = method
        if pqP is not None:
            # density-fitted CCD (jues_cc_create_df)
            if method != 0:
                raise ValueError("density fitting is built for CCD only")
            b, J = df_arrays(pqP, Jpqh)
            _lib.check(self.ctx.lib.jues_cc_create_df(self.ctx.h, b.ctypes.data_as(C.c_void_p), 0, n, b.shape[2],
                                                      _lib.ptr(J), _lib.ptr(Co), self.o, _lib.ptr(Cv), self.v,
                                                      _lib.ptr(e), C.byref(self.opts),
                                                      _lib.DF_VARIANT[df_variant], C.byref(h)))
            self.h = h
            return
        if gao_dev_ptr is not None:
            gp, isdev = C.c_void_p(gao_dev_ptr), 1
        else:
            self._g = _lib.f64(gao)
            gp, isdev = self._g.ctypes.data_as(C.c_void_p), 0
        _lib.check(self.ctx.lib.jues_cc_create(self.ctx.h, method, gp, isdev, n, _lib.ptr(Co),
                                               self.o, _lib.ptr(Cv), self.v, _lib.ptr(e),
                                               C.byref(self.opts), C.byref(h)))
        self._g = None
        self.h = h
        self.method = method

    def iterate(self, nsweeps=1):
        done = C.c_int()
        conv = C.c_int()
        _lib.check(self.ctx.lib.jues_cc_iterate(self.h, nsweeps, C.byref(done), C.byref(conv)))
        return done.value, bool(conv.value)

    def set_precision(self, precision):
        _lib.check(self.ctx.lib.jues_cc_set_precision(self.h, _lib.PREC[precision]))

    def energy(self):
        e = C.c_double()
        _lib.check(self.ctx.lib.jues_cc_energy(self.h, C.byref(e)))
        return e.value

    def amplitudes(self):
        T2 = np.empty((self.o, self.o, self.v, self.v), order="F")
        t1 = np.empty((self.o, self.v), order="F")
        _lib.check(self.ctx.lib.jues_cc_amplitudes(self.h, _lib.ptr(t1), _lib.ptr(T2)))
        return t1, T2

    def pT(self, precision="fp64"):
        """(T) correction on the session's CCSD amplitudes (jues_cc_pT)."""
        e = C.c_double()
        _lib.check(self.ctx.lib.jues_cc_pT(self.h, _lib.PREC[precision], C.byref(e)))
        return e.value

    def log(self):
        cnt = C.c_int()
        _lib.check(self.ctx.lib.jues_cc_log(self.h, None, 0, C.byref(cnt)))
        buf = (_lib.IterLog * max(1, cnt.value))()
        _lib.check(self.ctx.lib.jues_cc_log(self.h, buf, cnt.value, C.byref(cnt)))
        return [(r.iter, r.energy, r.rnorm, r.ms, r.precision) for r in buf[: cnt.value]]

    def close(self):
        if self.h:
            self.ctx.lib.jues_cc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
