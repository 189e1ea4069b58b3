"""ctypes binding of libjuesgpu.so (the C ABI declared in include/jues_gpu.h).

There is no CPU fallback: if the shared library is missing or no GB300 is visible,
every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(HERE), "lib", "libjuesgpu.so")

OK, EINVAL, ENOMEM, ECUDA, ENOTCONV, ENONFINITE, ETIMEOUT, ENODEV = range(8)
# "split": the split form at <= 1 uEh (three integer planes for contractions that produce
# integrals, two for the CC sweeps); "split_bf16" is its earlier name.  "split3" / "split2":
# three / two planes everywhere.
PREC = {"fp64": 0, "split": 1, "split_bf16": 1, "split3": 2, "split2": 3}
GUESS = {"zero": 0, "mp2": 1, "ovov": 2}
# CCSD Fae t1 term: "rccsd" = <ma|ef> (RCCSD.jl:190), "mrccsd" = <me|af> (mRCCSD.jl:140)
CCSD_FAE = {"rccsd": 0, "mrccsd": 1}


class JuESError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class NotConverged(JuESError):
    pass


class CCOpts(C.Structure):
    _fields_ = [("maxit", C.c_int), ("e_conv", C.c_double), ("r_conv", C.c_double),
                ("diis", C.c_int), ("diis_size", C.c_int), ("precision", C.c_int),
                ("guess", C.c_int), ("refine", C.c_int), ("transform_precision", C.c_int),
                ("ccsd_fae", C.c_int)]


class IterLog(C.Structure):
    _fields_ = [("iter", C.c_int), ("precision", C.c_int), ("energy", C.c_double),
                ("rnorm", C.c_double), ("ms", C.c_double)]


class MP2System(C.Structure):
    _fields_ = [("n", C.c_int), ("o", C.c_int), ("gao", C.POINTER(C.c_double)),
                ("C", C.POINTER(C.c_double)), ("eps", C.POINTER(C.c_double))]


class BatchInfo(C.Structure):
    _fields_ = [("upload_ms", C.c_double), ("graph_ms", C.c_double), ("download_ms", C.c_double),
                ("graph_nodes", C.c_int), ("tuned", C.c_int), ("nstages", C.c_int),
                ("tile_shape", C.c_int * 16)]


DP = C.POINTER(C.c_double)
VP = C.c_void_p

# name -> (restype, argtypes)
DF_VARIANT = {"reference": 0, "rccd": 1}

SIGNATURES = {
    "jues_version": (C.c_int, []),
    "jues_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "jues_ctx_create": (C.c_int, [C.c_int, C.POINTER(VP)]),
    "jues_ctx_destroy": (C.c_int, [VP]),
    "jues_ctx_set_mem_limit": (C.c_int, [VP, C.c_size_t]),
    "jues_ctx_set_profiling": (C.c_int, [VP, C.c_int]),
    "jues_ctx_profile": (C.c_int, [VP, C.c_char_p, DP, C.POINTER(C.c_longlong)]),
    "jues_ctx_profile_reset": (C.c_int, [VP]),
    "jues_ctx_launch_count": (C.c_longlong, [VP]),
    "jues_gemm": (C.c_int, [VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, DP, C.c_int,
                            DP, C.c_int, C.c_double, DP, C.c_int, C.c_int]),
    "jues_debug_expired_wait": (C.c_int, [VP]),
    "jues_gemm_noalloc": (C.c_int, [VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, VP, C.c_int,
                                    VP, C.c_int, C.c_double, VP, C.c_int]),
    "jues_tei_transform": (C.c_int, [VP, DP, C.c_int, DP, C.c_int, DP, C.c_int, DP, C.c_int, DP,
                                     C.c_int, C.c_int, DP]),
    "jues_get_eri": (C.c_int, [VP, DP, C.c_int, DP, C.c_int, DP, C.c_int, C.c_char_p, C.c_int,
                               C.c_int, C.c_int, DP]),
    "jues_rmp2": (C.c_int, [VP, DP, C.c_int, DP, C.c_int, DP, C.c_int, DP, C.c_int, DP, DP]),
    "jues_df_rmp2": (C.c_int, [VP, DP, C.c_int, C.c_int, DP, DP, C.c_int, DP, C.c_int, DP, C.c_int, DP]),
    "jues_rmp2_adjoint": (C.c_int, [VP, DP, C.c_int, DP, C.c_int, DP, C.c_int, C.c_double, DP, DP, DP]),
    "jues_batch_rmp2": (C.c_int, [VP, C.c_int, C.POINTER(MP2System), C.c_int, C.c_double, DP, C.POINTER(DP),
                                  C.POINTER(DP), C.POINTER(BatchInfo)]),
    "jues_cc_default_opts": (C.c_int, [C.POINTER(CCOpts)]),
    "jues_rccd": (C.c_int, [VP, DP, C.c_int, DP, C.c_int, DP, C.c_int, DP, C.POINTER(CCOpts), DP,
                            DP, C.POINTER(IterLog), C.c_int, C.POINTER(C.c_int)]),
    "jues_rccsd": (C.c_int, [VP, DP, C.c_int, DP, C.c_int, DP, C.c_int, DP, C.POINTER(CCOpts), DP,
                             DP, DP, C.POINTER(IterLog), C.c_int, C.POINTER(C.c_int)]),
    "jues_cc_create": (C.c_int, [VP, C.c_int, VP, C.c_int, C.c_int, DP, C.c_int, DP, C.c_int, DP,
                                 C.POINTER(CCOpts), C.POINTER(VP)]),
    "jues_cc_create_df": (C.c_int, [VP, VP, C.c_int, C.c_int, C.c_int, DP, DP, C.c_int, DP, C.c_int, DP,
                                    C.POINTER(CCOpts), C.c_int, C.POINTER(VP)]),
    "jues_df_rccd": (C.c_int, [VP, DP, C.c_int, C.c_int, DP, DP, C.c_int, DP, C.c_int, DP, C.POINTER(CCOpts),
                               C.c_int, DP, DP, C.POINTER(IterLog), C.c_int, C.POINTER(C.c_int)]),
    "jues_pT": (C.c_int, [VP, DP, DP, DP, DP, DP, DP, DP, C.c_int, C.c_int, C.c_int, DP]),
    "jues_get_fock": (C.c_int, [VP, DP, DP, C.c_int, DP, C.c_int, C.c_int, DP]),
    "jues_auto_rccsd": (C.c_int, [VP, DP, DP, C.c_int, DP, C.c_int, C.c_int, C.c_int, C.POINTER(CCOpts), C.c_int,
                                  DP, DP, DP, DP, C.POINTER(IterLog), C.c_int, C.POINTER(C.c_int)]),
    "jues_cc_pT": (C.c_int, [VP, C.c_int, DP]),
    "jues_ctx_set_ao_direct": (C.c_int, [VP, C.c_int, C.POINTER(C.c_int)]),
    "jues_ctx_set_batch_form": (C.c_int, [VP, C.c_int]),
    "jues_cc_iterate": (C.c_int, [VP, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "jues_cc_set_precision": (C.c_int, [VP, C.c_int]),
    "jues_cc_energy": (C.c_int, [VP, DP]),
    "jues_cc_amplitudes": (C.c_int, [VP, DP, DP]),
    "jues_cc_log": (C.c_int, [VP, C.POINTER(IterLog), C.c_int, C.POINTER(C.c_int)]),
    "jues_cc_destroy": (C.c_int, [VP]),
}

_lib = None
_lock = threading.Lock()
_ctxs = {}


def load(path: Optional[str] = None):
    """Load libjuesgpu.so and bind every C ABI symbol (no GPU needed)."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise JuESError(ENODEV, f"{p} is not built; run __graft_entry__.build() or "
                                    "python jues.jl_gb300/build.py")
        lib = C.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def last_error() -> str:
    buf = C.create_string_buffer(4096)
    load().jues_last_error(buf, 4096)
    return buf.value.decode(errors="replace")


def check(code: int):
    if code == OK:
        return
    msg = last_error()
    if code == ENOTCONV:
        raise NotConverged(code, msg)
    raise JuESError(code, msg)


class Context:
    """A device context (stream + memory) of the library."""

    def __init__(self, device: int = 0):
        lib = load()
        h = VP()
        check(lib.jues_ctx_create(device, C.byref(h)))
        self.h = h
        self.device = device
        self.lib = lib

    def close(self):
        if self.h:
            self.lib.jues_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_mem_limit(self, nbytes: int):
        check(self.lib.jues_ctx_set_mem_limit(self.h, nbytes))

    def set_profiling(self, on: bool):
        check(self.lib.jues_ctx_set_profiling(self.h, 1 if on else 0))

    def profile(self, prefix: str):
        t = C.c_double()
        n = C.c_longlong()
        check(self.lib.jues_ctx_profile(self.h, prefix.encode(), C.byref(t), C.byref(n)))
        return t.value, n.value

    def profile_reset(self):
        check(self.lib.jues_ctx_profile_reset(self.h))

    def set_ao_direct(self, enable: bool) -> bool:
        """Read host AO integrals in place where the device supports it; returns whether on."""
        a = C.c_int()
        check(self.lib.jues_ctx_set_ao_direct(self.h, 1 if enable else 0, C.byref(a)))
        return bool(a.value)

    def set_batch_form(self, form: str):
        """Forms the batched MP2 autotuning may pick: "auto", "fp64" or "tcgen05"."""
        check(self.lib.jues_ctx_set_batch_form(self.h, {"auto": 0, "fp64": 1, "tcgen05": 2}[form]))

    def launches(self) -> int:
        return int(self.lib.jues_ctx_launch_count(self.h))


def context(device: int = 0) -> Context:
    c = _ctxs.get(device)
    if c is None or c.h is None:
        c = Context(device)
        _ctxs[device] = c
    return c


def f64(x) -> np.ndarray:
    """Column-major float64 view/copy (Julia layout); Float32 inputs are promoted."""
    return np.asfortranarray(np.asarray(x, dtype=np.float64))


def ptr(a: Optional[np.ndarray]):
    if a is None:
        return None
    return a.ctypes.data_as(DP)


def gemm(A, B, C=None, alpha=1.0, beta=0.0, transA=False, transB=False, precision="fp64",
         device=0) -> np.ndarray:
    """C = alpha op(A) op(B) + beta C on the GPU (column-major, like BLAS.gemm!)."""
    A = f64(A)
    B = f64(B)
    M = A.shape[1] if transA else A.shape[0]
    K = A.shape[0] if transA else A.shape[1]
    N = B.shape[0] if transB else B.shape[1]
    if (B.shape[1] if transB else B.shape[0]) != K:
        raise ValueError("inner dimensions differ")
    Cm = np.zeros((M, N), order="F") if C is None else f64(C).copy(order="F")
    ctx = context(device)
    check(ctx.lib.jues_gemm(ctx.h, int(transA), int(transB), M, N, K, alpha, ptr(A), max(1, A.shape[0]),
                            ptr(B), max(1, B.shape[0]), beta, ptr(Cm), max(1, M), PREC[precision]))
    return Cm


def default_opts() -> CCOpts:
    o = CCOpts()
    check(load().jues_cc_default_opts(C.byref(o)))
    return o
