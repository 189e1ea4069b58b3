"""The allocation-free split GEMM (jues_gemm_noalloc) against the allocating entry point.

jues_gemm_noalloc exists for callers that cannot allocate device memory when they contract
(work running under CUDA graph capture, hosts whose device memory belongs to their own pool,
fixed-budget callers): it packs into a static device array instead.  The caller owns the
device buffers, here created with torch.  Two calls in a row check that the shared array is
fully rewritten by each call; the result must match the allocating entry point within the
1e-6 (of max |C|) bar the split-GEMM tests use.  Collected last on purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, X):
    # column-major X as a device buffer: X^T in C order has X's column-major bytes
    return torch.from_numpy(np.ascontiguousarray(np.asarray(X, dtype=np.float64).T)).cuda()


def test_noalloc_gemm_matches_allocating_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from juesgpu import _lib
    ctx = _lib.context(0)
    rng = np.random.default_rng(11)
    cases = [(300, 200, 500, False, True), (257, 129, 1000, True, False)]
    for M, N, K, ta, tb in cases:
        A = rng.normal(size=(K, M) if ta else (M, K))
        B = rng.normal(size=(N, K) if tb else (K, N))
        C0 = rng.normal(size=(M, N))
        want = _lib.gemm(A, B, C0, alpha=0.5, beta=2.0, transA=ta, transB=tb, precision="split_bf16")
        dA, dB, dC = _dev(torch, A), _dev(torch, B), _dev(torch, C0)
        torch.cuda.synchronize()
        st = ctx.lib.jues_gemm_noalloc(ctx.h, int(ta), int(tb), M, N, K, 0.5, dA.data_ptr(), A.shape[0],
                                       dB.data_ptr(), B.shape[0], 2.0, dC.data_ptr(), M)
        _lib.check(st)
        got = dC.cpu().numpy().T
        assert got.shape == (M, N)
        assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()


def test_noalloc_gemm_rejects_problems_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from juesgpu import _lib
    ctx = _lib.context(0)
    d = torch.zeros(16, dtype=torch.float64, device="cuda")   # never read: the size check comes first
    n = 4096   # packed operands 4 * (4096 + 4096) * 4096 bytes = 128 MiB > 64 MiB
    st = ctx.lib.jues_gemm_noalloc(ctx.h, 0, 0, n, n, n, 1.0, d.data_ptr(), n, d.data_ptr(), n, 0.0,
                                   d.data_ptr(), n)
    assert st == _lib.EINVAL
    assert "static scratch" in _lib.last_error()
