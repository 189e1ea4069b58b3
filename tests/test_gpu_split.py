"""GPU checks of the split-BF16 (tcgen05) form.

Bars: against an exact emulation of the operand representation (power-of-two fixed point per
row and 128-long K chunk, hi + lo/1024 carried in FP16, three products) the kernel may differ
only by the round-to-nearest FP32 sum of its chunk sums (1e-6 of max|C|); the relative Frobenius error against exact FP64
must stay below 1e-5 (~20 bits kept; a single BF16 product gives ~4e-3), also at K = 25600.
Energies: within 1 uEh of the FP64 oracle.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
import oracle
from juesgpu.synthetic import make_named, make_system

pytestmark = pytest.mark.gpu


KCH = 128
JUES_PREC_SPLIT = 1


def split_rows(X):
    """Integer-carrier split of each row of X over its columns (= K), chunk by chunk of 128:
    the library's operand representation x ~ 2^(e-9) (hi + lo/1024), |hi|, |lo| <= 512,
    with max |x| < 2^e over the chunk.  Returns hi, lo and the per-element exponent e."""
    X = np.asarray(X, dtype=np.float64)
    R, K = X.shape
    e = np.zeros_like(X, dtype=np.int64)
    for c0 in range(0, K, KCH):
        mx = np.abs(X[:, c0:c0 + KCH]).max(axis=1)
        e[:, c0:c0 + KCH] = np.where(mx > 0, np.frexp(mx)[1], 0)[:, None]
    # q = rint(x 2^(19-e)) with ties away from zero, hi = floor((q + 512) / 1024), lo = q - 1024 hi
    # (exactly the kernel's integer procedure; the scaling by 2^(19-e) is exact)
    t = np.ldexp(np.abs(X), 19 - e)
    q = np.sign(X) * np.floor(t + 0.5)
    h = np.floor((q + 512.0) / 1024.0)
    lo = q - 1024.0 * h
    return h, lo, e


def emulate(A, B):
    """Exact value of what the kernel computes for C = A @ B: per chunk, main + corr/1024 scaled
    by 2^(e_A + e_B - 18)."""
    ha, la, ea = split_rows(A)
    hb, lb, eb = split_rows(B.T)
    K = A.shape[1]
    C = np.zeros((A.shape[0], B.shape[1]))
    for c0 in range(0, K, KCH):
        s = slice(c0, c0 + KCH)
        main = ha[:, s] @ hb[:, s].T
        corr = ha[:, s] @ lb[:, s].T + la[:, s] @ hb[:, s].T
        C += np.ldexp(main + corr / 1024.0, ea[:, c0][:, None] + eb[:, c0][None, :] - 18)
    return C


@pytest.fixture(scope="module")
def lib():
    from juesgpu import _lib
    _lib.context(0)
    return _lib


SHAPES = [(128, 128, 64, False, False), (200, 72, 300, False, True), (1000, 257, 129, True, False),
          (77, 1000, 640, True, True), (4096, 300, 2000, False, False), (640, 64, 6400, False, False),
          (33, 4000, 513, False, True)]


@pytest.mark.parametrize("M,N,K,ta,tb", SHAPES)
def test_gemm_fp64(lib, M, N, K, ta, tb):
    rng = np.random.default_rng(M + N + K)
    A = rng.normal(size=(K, M) if ta else (M, K))
    B = rng.normal(size=(N, K) if tb else (K, N))
    C0 = rng.normal(size=(M, N))
    got = lib.gemm(A, B, C0, alpha=0.7, beta=-1.3, transA=ta, transB=tb)
    want = 0.7 * ((A.T if ta else A) @ (B.T if tb else B)) - 1.3 * C0
    assert np.allclose(got, want, rtol=1e-12, atol=1e-11 * np.sqrt(K))


def test_gemm_split_epilogue_forms(lib):
    """The epilogue's forms against the plain product P = gemm(A, B): alpha a power of two is
    folded into the FP32 scale (exact), other alphas multiply in FP64, beta = 1 adds in place
    (in L2), other betas read C.  All but the general beta are bit-exact images of P."""
    rng = np.random.default_rng(11)
    A = rng.normal(size=(1000, 129))
    B = rng.normal(size=(129, 257))
    C0 = rng.normal(size=(1000, 257))
    P = lib.gemm(A, B, precision="split_bf16")
    for alpha in (1.0, -0.5, 4.0, 0.7):
        assert np.array_equal(lib.gemm(A, B, alpha=alpha, precision="split_bf16"), alpha * P)
        assert np.array_equal(lib.gemm(A, B, C0, alpha=alpha, beta=1.0, precision="split_bf16"), C0 + alpha * P)
        got = lib.gemm(A, B, C0, alpha=alpha, beta=-1.3, precision="split_bf16")
        assert np.abs(got - (alpha * P - 1.3 * C0)).max() < 1e-14 * np.abs(got).max()


def test_gemm_split_ragged_last_round(lib):
    """160 output tiles on a GPU of ~150 SMs: the tiles of the ragged last round are split over K
    (FP32 parts summed in FP64 by a second kernel).  Every tile must match the exact emulation of
    the split representation, and the epilogue forms (alpha folded or not, beta = 1 in place,
    general beta) must hold on the split tiles as on the whole ones."""
    rng = np.random.default_rng(21)
    A = rng.normal(size=(20480, 1024))
    B = rng.normal(size=(1024, 128))
    C0 = rng.normal(size=(20480, 128))
    emu = emulate(A, B)
    P = lib.gemm(A, B, precision="split_bf16")
    assert np.abs(P - emu).max() < 1e-6 * np.abs(emu).max()
    # the tail rows (the last tiles) were computed by the split path
    assert np.abs(P[-1024:] - emu[-1024:]).max() < 1e-6 * np.abs(emu).max()
    for alpha, beta in ((-0.5, 1.0), (0.7, 1.0), (4.0, 0.0), (0.7, -1.3)):
        got = lib.gemm(A, B, C0, alpha=alpha, beta=beta, precision="split_bf16")
        want = alpha * emu + beta * C0
        assert np.abs(got - want).max() < 2e-6 * np.abs(want).max()


@pytest.mark.parametrize("M,N,K,ta,tb", SHAPES)
def test_gemm_split_bf16(lib, M, N, K, ta, tb):
    rng = np.random.default_rng(7 * M + N + K)
    A = rng.normal(size=(K, M) if ta else (M, K))
    B = rng.normal(size=(N, K) if tb else (K, N))
    C0 = rng.normal(size=(M, N))
    got = lib.gemm(A, B, C0, alpha=0.7, beta=-1.3, transA=ta, transB=tb, precision="split_bf16")
    Aop, Bop = (A.T if ta else A), (B.T if tb else B)
    emu = 0.7 * emulate(Aop, Bop) - 1.3 * C0
    exact = 0.7 * (Aop @ Bop) - 1.3 * C0
    scale = np.sqrt(K)
    # the kernel's chunk sums are exact; only the round-to-nearest FP32 sum of chunks and the
    # final FP64 rescale separate it from the exact three-product value
    assert np.abs(got - emu).max() < 1e-6 * np.abs(emu).max()
    ref = exact + 1.3 * C0
    rel = np.linalg.norm(got - exact) / np.linalg.norm(ref)
    assert rel < 1e-5


def test_gemm_split_bf16_long_k(lib):
    # K = 25600 is the pp-ladder's contraction length at nbf=200
    rng = np.random.default_rng(3)
    A = rng.normal(size=(256, 25600))
    B = rng.normal(size=(25600, 192))
    got = lib.gemm(A, B, precision="split_bf16")
    exact = A @ B
    assert np.linalg.norm(got - exact) / np.linalg.norm(exact) < 1e-5


def test_transform_split(lib):
    import juesgpu.Transformation as Tr
    s = make_system(48, 12, 144, seed=9)
    g = s.ao_eri()
    rng = np.random.default_rng(1)
    Cs = [s.C[:, :12], s.C[:, 12:], s.C[:, :12], s.C[:, 12:]]
    got = Tr.tei_transform(g, *Cs, precision="split_bf16")
    want = oracle.tei_transform(g, *Cs)
    assert np.abs(got - want).max() < 1e-4 * np.abs(want).max()


@pytest.mark.parametrize("name", ["S25", "S100"])
def test_rmp2_split(lib, name):
    from juesgpu import MollerPlesset
    with open(os.path.join(GOLDEN, "synthetic_golden.json")) as f:
        ref = json.load(f)[name]["mp2"]
    e = MollerPlesset.do_rmp2(make_named(name).wfn(), precision="split_bf16")
    assert abs(e - ref) < 1e-6


@pytest.mark.parametrize("refine,tprec", [(0, None), (2, "fp64")])
def test_rccd_split_within_one_microhartree(lib, refine, tprec):
    from juesgpu.CoupledCluster import mRCCD
    with open(os.path.join(GOLDEN, "synthetic_golden.json")) as f:
        ref = json.load(f)["S100"]["ccd_mp2guess_diis"]["energy"]
    w = make_named("S100").wfn()
    e, log = mRCCD.do_rccd(w, maxit=40, r_conv=1e-9, guess="mp2", precision="split_bf16",
                           refine=refine, transform_precision=tprec, return_log=True)
    assert abs(e - ref) < 1e-6, (e, ref, log)
    if refine:
        assert log[-1][4] == 0 and log[0][4] == 1      # closing sweeps ran in FP64


def test_rccsd_split(lib):
    from juesgpu.CoupledCluster import RCCSD
    with open(os.path.join(GOLDEN, "synthetic_golden.json")) as f:
        ref = json.load(f)["S25"]["ccsd_diis"]["energy"]
    e = RCCSD.do_rccsd(make_named("S25").wfn(), maxit=60, diis=True, r_conv=1e-9,
                       precision="split_bf16", refine=2)
    assert abs(e - ref) < 1e-6


@pytest.mark.parametrize("precision", ["fp64", "split_bf16"])
@pytest.mark.parametrize("M,N,K", [(40, 40, 200000), (160, 96, 64000), (300, 200, 4096)])
def test_gemm_split_k(lib, precision, M, N, K):
    # small outputs with long contractions (the Fmi / Fae intermediates) are split over K and
    # reduced in FP64; alpha, beta and a transposed operand go through the reduction epilogue
    rng = np.random.default_rng(M * N + K)
    A = rng.normal(size=(K, M))
    B = rng.normal(size=(K, N))
    C0 = rng.normal(size=(M, N))
    got = lib.gemm(A, B, C0, alpha=-0.5, beta=0.25, transA=True, precision=precision)
    exact = -0.5 * (A.T @ B) + 0.25 * C0
    if precision == "fp64":
        assert np.allclose(got, exact, rtol=1e-12, atol=1e-11 * np.sqrt(K))
    else:
        rel = np.linalg.norm(got - exact) / np.linalg.norm(0.5 * (A.T @ B))
        assert rel < 1e-5
    again = lib.gemm(A, B, C0, alpha=-0.5, beta=0.25, transA=True, precision=precision)
    assert np.array_equal(got, again)   # the split order is fixed: bitwise reproducible


# ------------------------------------------------------------------------------ three planes
def split3_rows(X):
    """The three-plane operand representation: q = rint(x 2^(29-e)) (ties away from zero) =
    2^20 hi + 2^10 mid + lo, each in [-512, 512], per row and 128-long K chunk."""
    X = np.asarray(X, dtype=np.float64)
    R, K = X.shape
    e = np.zeros_like(X, dtype=np.int64)
    for c0 in range(0, K, KCH):
        mx = np.abs(X[:, c0:c0 + KCH]).max(axis=1)
        e[:, c0:c0 + KCH] = np.where(mx > 0, np.frexp(mx)[1], 0)[:, None]
    t = np.ldexp(np.abs(X), 29 - e)
    q = np.sign(X) * np.floor(t + 0.5)
    h = np.floor((q + 2.0**19) / 2.0**20)
    rem = q - 2.0**20 * h
    m = np.floor((rem + 512.0) / 1024.0)
    lo = rem - 1024.0 * m
    return h, m, lo, e


def emulate3(A, B):
    """What the three-plane kernel computes, with its FP32 roundings: per chunk the exact
    integer accumulators main = hh, c1 = hm + mh, c2 = hl + mm + lh, then in FP32
    part = (c2 2^-10 + c1) 2^-10 + main and acc += part 2^(e_A + e_B - 18)."""
    ha, ma, la, ea = split3_rows(A)
    hb, mb, lb, eb = split3_rows(B.T)
    K = A.shape[1]
    f32 = np.float32
    acc = np.zeros((A.shape[0], B.shape[1]), dtype=f32)
    for c0 in range(0, K, KCH):
        s = slice(c0, c0 + KCH)
        main = ha[:, s] @ hb[:, s].T
        c1 = ha[:, s] @ mb[:, s].T + ma[:, s] @ hb[:, s].T
        c2 = ha[:, s] @ lb[:, s].T + ma[:, s] @ mb[:, s].T + la[:, s] @ hb[:, s].T
        corr = f32(c2 / 1024.0 + c1)
        part = f32(corr.astype(np.float64) / 1024.0 + main)
        sc = np.ldexp(1.0, ea[:, c0][:, None] + eb[:, c0][None, :] - 18)
        acc = f32(part.astype(np.float64) * sc + acc.astype(np.float64))
    return acc.astype(np.float64)


@pytest.mark.parametrize("M,N,K,ta,tb", SHAPES[:6])
def test_gemm_split3(lib, M, N, K, ta, tb):
    rng = np.random.default_rng(11 * M + N + K)
    A = rng.normal(size=(K, M) if ta else (M, K))
    B = rng.normal(size=(N, K) if tb else (K, N))
    got = lib.gemm(A, B, transA=ta, transB=tb, precision="split3")
    Aop, Bop = (A.T if ta else A), (B.T if tb else B)
    exact = Aop @ Bop
    emu = emulate3(Aop, Bop)
    # the FP32 roundings dominate: ~2^-24 per chunk sum, growing like sqrt(chunks)
    assert np.abs(got - emu).max() < 1e-6 * np.abs(exact).max()
    rel = np.linalg.norm(got - exact) / np.linalg.norm(exact)
    assert rel < (3e-7 if K <= 640 else 1e-6), rel
    # and far better than the two-plane form
    two = lib.gemm(A, B, transA=ta, transB=tb, precision="split_bf16")
    assert rel < 0.2 * np.linalg.norm(two - exact) / np.linalg.norm(exact)


@pytest.mark.parametrize("name,bar", [("S25", 1e-10), ("S100", 3e-8)])
def test_rmp2_split3(lib, name, bar):
    from juesgpu import MollerPlesset
    with open(os.path.join(GOLDEN, "synthetic_golden.json")) as f:
        ref = json.load(f)[name]["mp2"]
    e = MollerPlesset.do_rmp2(make_named(name).wfn(), precision="split3")
    assert abs(e - ref) < bar, (e, ref)


def test_rccd_split3_transform_within_one_microhartree(lib):
    # the microhartree setting without FP64 arithmetic: split3 integrals, split sweeps
    from juesgpu.CoupledCluster import mRCCD
    with open(os.path.join(GOLDEN, "synthetic_golden.json")) as f:
        ref = json.load(f)["S100"]["ccd_mp2guess_diis"]["energy"]
    w = make_named("S100").wfn()
    e, log = mRCCD.do_rccd(w, maxit=40, r_conv=1e-8, guess="mp2", precision="split_bf16", refine=0,
                           transform_precision="split3", return_log=True)
    assert abs(e - ref) < 1e-6, (e, ref)
    assert all(r[4] == 1 for r in log)


@pytest.mark.parametrize("name", ["S25", "S100"])
def test_ao_direct_matches_device_copy(lib, name):
    # split forms pack the host AO array in place where the device reads pageable memory through
    # the host page tables; the packed values, hence the results, are the same bits as after a
    # device copy
    from juesgpu import MollerPlesset
    from juesgpu.CoupledCluster import mRCCD
    ctx = lib.context(0)
    w = make_named(name).wfn()
    on = ctx.set_ao_direct(True)
    e1 = MollerPlesset.do_rmp2(w, precision="split_bf16")
    c1 = mRCCD.do_rccd(w, maxit=3, r_conv=0.0, guess="mp2", precision="split_bf16", refine=0)
    ctx.set_ao_direct(False)
    e2 = MollerPlesset.do_rmp2(w, precision="split_bf16")
    c2 = mRCCD.do_rccd(w, maxit=3, r_conv=0.0, guess="mp2", precision="split_bf16", refine=0)
    ctx.set_ao_direct(on)
    assert e1 == e2 and c1 == c2, (on, e1, e2, c1, c2)


def test_pack_cache_never_serves_a_freed_address(lib):
    # split operands are cached by source address and device memory is reused at once by the
    # context's pool: a session after another in the same context must give the bits of a
    # session in a fresh context
    from juesgpu import _lib
    from juesgpu.CoupledCluster import mRCCD
    w = make_named("S100").wfn()
    kw = dict(maxit=4, r_conv=0.0, guess="mp2", precision="split_bf16", refine=0)
    mRCCD.do_rccd(w, transform_precision="fp64", **kw)
    e_after = mRCCD.do_rccd(w, transform_precision="split3", **kw)
    saved = _lib._ctxs.get(0)
    fresh = _lib.Context(0)
    _lib._ctxs[0] = fresh
    try:
        e_fresh = mRCCD.do_rccd(w, transform_precision="split3", **kw)
    finally:
        _lib._ctxs[0] = saved
        fresh.close()
    assert e_after == e_fresh, (e_after, e_fresh)


# ------------------------------------------------------------------------------ nbf = 200
@pytest.fixture(scope="module")
def s200():
    return make_named("S200").wfn()


def test_rmp2_default_split_s200_within_one_microhartree(lib, s200):
    # the default split form keeps three planes in the transform: <= 1 uEh at the headline size
    # (two planes, the opt-in "split2", gave -4.8e-6 Eh here)
    from juesgpu import MollerPlesset
    ref = json.load(open(os.path.join(GOLDEN, "synthetic_golden.json")))["S200"]["mp2"]
    e = MollerPlesset.do_rmp2(s200, precision="split")
    assert abs(e - ref) < 1e-6, (e, ref)


def test_rccd_default_split_s200_converged_within_one_microhartree(lib, s200):
    # the configuration the bench times: three-plane integrals, two-plane sweeps, no FP64 sweep,
    # stopped at |dE| < 1e-7 Eh; against the FP64 oracle's converged energy
    from juesgpu.CoupledCluster import mRCCD
    ref = json.load(open(os.path.join(GOLDEN, "synthetic_golden.json")))["S200"]["ccd_mp2guess_diis"]["energy"]
    e, log = mRCCD.do_rccd(s200, maxit=60, r_conv=0.0, e_conv=1e-7, guess="mp2", precision="split", refine=0,
                           return_log=True)
    assert len(log) < 60 and all(r[4] == JUES_PREC_SPLIT for r in log)
    assert abs(e - ref) < 1e-6, (e, ref, len(log))


@pytest.mark.parametrize("method,name", [(0, "S25"), (0, "S100"), (1, "S25"), (1, "S100")])
def test_one_split_sweep_against_fp64_sweep(lib, method, name):
    # One sweep in split precision and one in FP64 from the same amplitudes (two FP64 sweeps from
    # the MP2 guess, so T2 is pair-symmetric and t1 nonzero) on the same FP64 integrals.  The
    # split sweep runs its ring contractions K-stacked (two GEMMs of K = 2 ov); its amplitudes
    # must agree with the FP64 sweep's to the split arithmetic's ~1e-6 of max|T| and the energy
    # to 1e-8 Eh, where any misplaced term would be >= 1e-3.
    from juesgpu.CoupledCluster import CCSession
    w = make_named(name).wfn()
    kw = dict(guess="mp2", diis=False, r_conv=0.0, maxit=10, transform_precision="fp64")
    ref = CCSession(method, w, precision="fp64", **kw)
    ses = CCSession(method, w, precision="split_bf16", **kw)
    ses.set_precision("fp64")
    ref.iterate(2)
    ses.iterate(2)
    t1a, Ta = ref.amplitudes()
    t1b, Tb = ses.amplitudes()
    assert np.array_equal(Ta, Tb)
    ref.iterate(1)
    ses.set_precision("split_bf16")
    ses.iterate(1)
    t1a, Ta = ref.amplitudes()
    t1b, Tb = ses.amplitudes()
    scale = np.abs(Ta).max()
    assert np.abs(Tb - Ta).max() < 3e-6 * scale, np.abs(Tb - Ta).max() / scale
    if method == 1:
        # t1 is a small sum of larger cancelling terms: its bar is relative to max|T2|
        assert np.abs(t1b - t1a).max() < 3e-6 * scale, np.abs(t1b - t1a).max() / scale
    assert abs(ses.energy() - ref.energy()) < 1e-8
    ref.close()
    ses.close()
