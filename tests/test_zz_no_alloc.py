"""The allocation-free split GEMM (jues_gemm_noalloc) on caller-owned device buffers.

jues_gemm_noalloc exists for callers that cannot let the library allocate device memory when
they contract (hosts that hand out the GPU's memory from their own pool, fixed-budget
services): it packs into a static device array instead.  The caller owns the device buffers,
here created with torch.  Two calls in a row check that the shared array is fully rewritten by
each call.  Each result is compared with the exact FP64 value alpha op(A) op(B) + beta C0 at the
split-GEMM bar (relative Frobenius error 1e-5 of the product term) and with the allocating entry
point jues_gemm, which runs the same two-plane arithmetic (1e-6 of max |C|).  Collected last on
purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, X):
    # column-major X as a device buffer: X^T in C order has X's column-major bytes
    return torch.from_numpy(np.ascontiguousarray(np.asarray(X, dtype=np.float64).T)).cuda()


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def _noalloc(ctx, torch, A, B, C0, alpha, beta, ta, tb):
    from juesgpu import _lib
    M, N = C0.shape
    K = A.shape[0] if ta else A.shape[1]
    # an empty operand is never read; a one-element buffer stands in for its pointer
    dA = _dev(torch, A) if A.size else torch.zeros(1, dtype=torch.float64, device="cuda")
    dB = _dev(torch, B) if B.size else torch.zeros(1, dtype=torch.float64, device="cuda")
    dC = _dev(torch, C0)
    torch.cuda.synchronize()
    st = ctx.lib.jues_gemm_noalloc(ctx.h, int(ta), int(tb), M, N, K, alpha, dA.data_ptr(), max(1, A.shape[0]),
                                   dB.data_ptr(), max(1, B.shape[0]), beta, dC.data_ptr(), M)
    _lib.check(st)
    return dC.cpu().numpy().T


def test_noalloc_gemm_matches_fp64_product_on_two_calls():
    torch = _torch()
    from juesgpu import _lib
    ctx = _lib.context(0)
    rng = np.random.default_rng(11)
    cases = [(300, 200, 500, False, True), (257, 129, 1000, True, False)]
    for M, N, K, ta, tb in cases:
        A = rng.normal(size=(K, M) if ta else (M, K))
        B = rng.normal(size=(N, K) if tb else (K, N))
        C0 = rng.normal(size=(M, N))
        prod = (A.T if ta else A) @ (B.T if tb else B)
        exact = 0.5 * prod + 2.0 * C0
        alloc = _lib.gemm(A, B, C0, alpha=0.5, beta=2.0, transA=ta, transB=tb, precision="split")
        for call in range(2):
            got = _noalloc(ctx, torch, A, B, C0, 0.5, 2.0, ta, tb)
            assert got.shape == (M, N)
            rel = np.linalg.norm(got - exact) / np.linalg.norm(0.5 * prod)
            assert rel < 1e-5, (M, N, K, call, rel)
            assert np.abs(got - alloc).max() <= 1e-6 * np.abs(alloc).max(), (M, N, K, call)


def test_noalloc_gemm_empty_contraction_scales_c():
    # K = 0: the product is empty, C = beta C (beta = 0 writes zeros)
    torch = _torch()
    from juesgpu import _lib
    ctx = _lib.context(0)
    rng = np.random.default_rng(5)
    C0 = rng.normal(size=(37, 19))
    A = np.zeros((37, 0))
    B = np.zeros((0, 19))
    for beta in (-1.5, 0.0):
        got = _noalloc(ctx, torch, A, B, C0, 0.7, beta, False, False)
        assert np.array_equal(got, beta * C0 if beta else np.zeros_like(C0))


def test_noalloc_gemm_rejects_problems_beyond_its_scratch():
    torch = _torch()
    from juesgpu import _lib
    ctx = _lib.context(0)
    d = torch.zeros(16, dtype=torch.float64, device="cuda")   # never read: the size check comes first
    n = 4096   # packed operands 4 * (4096 + 4096) * 4096 bytes = 128 MiB > 64 MiB
    st = ctx.lib.jues_gemm_noalloc(ctx.h, 0, 0, n, n, n, 1.0, d.data_ptr(), n, d.data_ptr(), n, 0.0,
                                   d.data_ptr(), n)
    assert st == _lib.EINVAL
    assert "static scratch" in _lib.last_error()
