"""Bounded CPU timing samples of the reference's RCCD sweep (oracle; test infrastructure).

One full RCCD.jl sweep at nbf=200 takes minutes on a CPU, so the CPU baseline times 1/s of it
per step: every intermediate of RCCD.jl:169-467 is contracted over one slice of its last
virtual index (a partial sum, 1/s of its flops) and every term of the T2 update
(RCCD.jl:242-256) is formed for one slice of output columns b (using full intermediates
prepared before timing).  The s slices together are exactly one sweep's arithmetic, so
(step time) x s estimates the time per sweep.  Contractions run through numpy.einsum with
BLAS-backed pairwise contraction, the same permute + GEMM strategy as TensorOperations.
"""
import time

import numpy as np

E = lambda s, *ops: np.einsum(s, *ops, optimize=True)  # noqa: E731


class SlicedSweep:
    def __init__(self, oovv, ovov, ovvo, oooo, vvvv, eps, o, slices=16):
        self.o = o
        self.v = oovv.shape[2]
        self.s = slices
        self.ints = (oovv, ovov, ovvo, oooo, vvvv)
        ev = eps[o:]
        eo = eps[:o]
        self.D = (eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None]
                  - ev[None, None, None, :])
        self.T = oovv / self.D
        v = self.v
        # full intermediates with the reference's shapes; their values do not change the
        # arithmetic timed, so they are filled with a constant instead of being formed
        self.Fae = np.full((v, v), 1e-3)
        self.Fmi = np.full((o, o), 1e-3)
        self.Wmnij = np.full((o, o, o, o), 1e-3)
        self.Wabef = np.full((v, v, v, v), 1e-3)
        self.WmBeJ = np.full((o, v, v, o), 1e-3)
        self.WmBEj = np.full((o, v, v, o), 1e-3)
        bounds = np.linspace(0, v, slices + 1).astype(int)
        self.sl = [slice(bounds[k], bounds[k + 1]) for k in range(slices)]

    def step(self, k):
        """The k-th 1/s share of one sweep; returns the elapsed seconds."""
        oovv, ovov, ovvo, oooo, vvvv = self.ints
        T = self.T
        f = self.sl[k % self.s]
        t0 = time.perf_counter()
        Tt = 2 * T[:, :, :, f] - np.transpose(T, (1, 0, 2, 3))[:, :, :, f]
        # intermediates: contraction index f restricted to the slice (partial sums)
        E("mnef,mnaf->ae", oovv[:, :, :, f], Tt)
        E("mnef,inef->mi", oovv[:, :, :, f], (2 * T - np.transpose(T, (0, 1, 3, 2)))[:, :, :, f])
        E("ijef,mnef->mnij", T[:, :, :, f], oovv[:, :, :, f])
        E("mnab,mnef->abef", T, oovv[:, :, :, f])
        Tj = 2 * T - np.transpose(T, (1, 0, 2, 3))
        E("mnef,njfb->mbej", oovv[:, :, :, f], Tj[:, :, f, :])
        E("nmef,njfb->mbej", oovv[:, :, :, f], T[:, :, f, :])
        E("jnfb,nmef->mbej", T[:, :, f, :], oovv[:, :, :, f])
        # T2 update for output columns b in the slice
        b = f
        Fae, Fmi, Wmnij, Wabef, WJ, WK = (self.Fae, self.Fmi, self.Wmnij, self.Wabef, self.WmBeJ,
                                          self.WmBEj)
        R = (oovv[:, :, :, b] + E("ijae,be->ijab", T, Fae[b])
             + E("jibe,ae->ijab", T[:, :, b, :], Fae)
             - E("imab,mj->ijab", T[:, :, :, b], Fmi) - E("mjab,mi->ijab", T[:, :, :, b], Fmi)
             + E("mnab,mnij->ijab", T[:, :, :, b], Wmnij)
             + E("ijef,abef->ijab", T, Wabef[:, b])
             + 2 * E("imae,mbej->ijab", T, WJ[:, b]) - E("miae,mbej->ijab", T, WJ[:, b])
             + E("imae,mbej->ijab", T, WK[:, b]) + E("mibe,maej->ijab", T[:, :, b, :], WK)
             + E("mjae,mbei->ijab", T, WK[:, b]) + 2 * E("jmbe,maei->ijab", T[:, :, b, :], WJ)
             - E("mjbe,maei->ijab", T[:, :, b, :], WJ) + E("jmbe,maei->ijab", T[:, :, b, :], WK))
        R /= self.D[:, :, :, b]
        return time.perf_counter() - t0
