"""The reference's RCCD sweep cut into bounded CPU timing steps (oracle; test infrastructure).

One RCCD.jl sweep at nbf=200 takes tens of seconds on a CPU, so the CPU baseline times it in
STAGES steps of real work that carry their state from step to step:

* stage 0 forms Fae, Fmi and Wmnij (RCCD.jl:169-232, 312-341), and stages 0..NB-1 each form
  one slice of the last virtual index of Wabef (RCCD.jl:350-380), WmBeJ and WmBEj
  (RCCD.jl:390-467), from the current amplitudes;
* stages NB..2NB-1 each form one slice of output columns b of the T2 update (all fourteen terms
  of RCCD.jl:242-256, divided by D) from the complete intermediates;
* the last stage also swaps in the new amplitudes and evaluates the energy (RCCD.jl:99-117).

STAGES consecutive steps are exactly one RCCD.jl sweep, Jacobi update and energy included
(RCCD.do_rccd runs no DIIS), so the sum of their times is the measured time of one sweep.
Contractions run through numpy.einsum with BLAS-backed pairwise contraction, the same
permute + GEMM strategy as TensorOperations.
"""
import time

import numpy as np

E = lambda s, *ops: np.einsum(s, *ops, optimize=True)  # noqa: E731


class PipelinedSweep:
    """RCCD.jl sweeps as a sequence of stages; ``step()`` runs the next stage."""

    def __init__(self, oovv, ovov, ovvo, oooo, vvvv, eps, o, stages=16, guess="ovov"):
        if stages % 2:
            raise ValueError("stages must be even (half intermediates, half T2 update)")
        self.o = o
        self.v = v = oovv.shape[2]
        self.ints = (oovv, ovov, ovvo, oooo, vvvv)
        ev, eo = eps[o:], eps[:o]
        self.D = (eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None]
                  - ev[None, None, None, :])
        if guess == "ovov":            # RCCD.jl:145-160: T2 = ovov[i,a,j,b] / D
            self.T = np.transpose(ovov, (0, 2, 1, 3)) / self.D
        else:                          # the MP2 amplitudes
            self.T = oovv / self.D
        self.nb = stages // 2
        self.stages = stages
        bounds = np.linspace(0, v, self.nb + 1).astype(int)
        self.sl = [slice(bounds[k], bounds[k + 1]) for k in range(self.nb)]
        # intermediates, filled slice by slice
        self.Wabef = np.empty((v, v, v, v))
        self.WJ = np.empty((o, v, v, o))
        self.WK = np.empty((o, v, v, o))
        self.Tn = np.empty_like(self.T)
        self.k = 0            # next stage
        self.sweeps = 0       # completed sweeps
        self.energy = self.ccenergy(self.T)

    def ccenergy(self, T):
        oovv = self.ints[0]
        return float(np.sum(oovv * (2.0 * T - np.transpose(T, (1, 0, 2, 3)))))   # RCCD.jl:99-117

    def _intermediates(self, s):
        oovv, ovov, ovvo, oooo, vvvv = self.ints
        T = self.T
        f = self.sl[s]
        if s == 0:
            Tt = 2 * T - np.transpose(T, (1, 0, 2, 3))
            self.Fae = -E("mnef,mnaf->ae", oovv, Tt)                                   # RCCD.jl:179
            self.Fmi = E("mnef,inef->mi", oovv, 2 * T - np.transpose(T, (0, 1, 3, 2)))  # RCCD.jl:216
            self.Wmnij = oooo + E("ijef,mnef->mnij", T, oovv) / 2                       # RCCD.jl:320
            self.Tj = Tt
        # Wabef[a,b,e,f] for f in the slice (RCCD.jl:358)
        self.Wabef[:, :, :, f] = vvvv[:, :, :, f] + E("mnab,mnef->abef", T, oovv[:, :, :, f]) / 2
        # WmBeJ[m,b,e,j] and WmBEj[m,b,e,j] for b in the slice (RCCD.jl:400, 445)
        b = f
        self.WJ[:, b] = (ovvo[:, b] + E("mnef,njfb->mbej", oovv, self.Tj[:, :, :, b]) / 2
                         - E("nmef,njfb->mbej", oovv, T[:, :, :, b]) / 2)
        self.WK[:, b] = (-np.transpose(ovov[:, b], (0, 1, 3, 2))
                         + E("jnfb,nmef->mbej", T[:, :, :, b], oovv) / 2)

    def _update(self, s):
        oovv = self.ints[0]
        T, Fae, Fmi, Wmnij, Wabef, WJ, WK = (self.T, self.Fae, self.Fmi, self.Wmnij, self.Wabef,
                                             self.WJ, self.WK)
        b = self.sl[s]
        # RCCD.jl:242-256 for output columns b
        R = (oovv[:, :, :, b] + E("ijae,be->ijab", T, Fae[b])
             + E("jibe,ae->ijab", T[:, :, b, :], Fae)
             - E("imab,mj->ijab", T[:, :, :, b], Fmi) - E("mjab,mi->ijab", T[:, :, :, b], Fmi)
             + E("mnab,mnij->ijab", T[:, :, :, b], Wmnij)
             + E("ijef,abef->ijab", T, Wabef[:, b])
             + 2 * E("imae,mbej->ijab", T, WJ[:, b]) - E("miae,mbej->ijab", T, WJ[:, b])
             + E("imae,mbej->ijab", T, WK[:, b]) + E("mibe,maej->ijab", T[:, :, b, :], WK)
             + E("mjae,mbei->ijab", T, WK[:, b]) + 2 * E("jmbe,maei->ijab", T[:, :, b, :], WJ)
             - E("mjbe,maei->ijab", T[:, :, b, :], WJ) + E("jmbe,maei->ijab", T[:, :, b, :], WK))
        self.Tn[:, :, :, b] = R / self.D[:, :, :, b]

    def step(self):
        """Run the next stage; returns (stage index, elapsed seconds)."""
        k = self.k
        t0 = time.perf_counter()
        if k < self.nb:
            self._intermediates(k)
        else:
            self._update(k - self.nb)
            if k == self.stages - 1:
                self.T, self.Tn = self.Tn, self.T
                self.energy = self.ccenergy(self.T)
                self.sweeps += 1
        dt = time.perf_counter() - t0
        self.k = (k + 1) % self.stages
        return k, dt
