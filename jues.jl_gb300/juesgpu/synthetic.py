"""Seeded synthetic closed-shell systems (the workload generator).

The reference is driven by molecular integrals from libint/psi4, which are not
available here; the benchmarks and parity tests run on synthetic systems whose
AO integrals are exactly B-factored, hence 8-fold symmetric and positive
semi-definite like real ERIs::

    (mu nu|lambda sigma) = sum_P B[P,mu,nu] * B[P,lambda,sigma]

Draw order (numpy PCG64 ``default_rng(seed)``), fixed so that every consumer
reads identical bytes:

1. ``B``: for P = 0..naux-1 the upper triangle (mu <= nu, row-major) is drawn
   from N(0, sigma^2) and mirrored.
2. ``G`` ~ N(0,1), n x n; ``C, _ = numpy.linalg.qr(G)`` (orthonormal AO basis).
3. occupied energies ~ U[-2.0,-0.5] (o draws), virtual ~ U[0.2,3.0] (v draws),
   each sorted ascending; ``eps = [occ; vir]``.
4. ``H = (X + X^T)/sqrt(2)`` with X ~ N(0, 0.5^2) (one-electron matrix; not read
   by the hot path).

sigma: the literal N(0, 0.1^2) entries make (ia|ia) ~ 0.01*naux, i.e. MP2
amplitudes of order one, and coupled-cluster iterations diverge for every size
(measured: E_MP2 = -38.7 Eh at nbf=25, -27900 Eh at nbf=100, CCD overflowing
after ~30 DIIS steps).  The default therefore scales the entries as
``sigma = 0.15/sqrt(naux)``, which keeps (ia|ia) = O(0.02) at every size and gives
CC problems that converge to 1e-10 in the 10-30 iterations a real molecule
needs.  ``sigma=0.1`` reproduces the literal distribution.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np

from .Wavefunction import Wfn, wfn_from_rhf

# name -> (nbf, nocc, naux)
SHAPES = {
    "S25": (25, 5, 75),
    "S100": (100, 20, 300),
    "S200": (200, 40, 600),
    "ADJ120": (120, 25, 360),
}

DEFAULT_B_SCALE = 0.15


@dataclass
class SyntheticSystem:
    nbf: int
    nocc: int
    naux: int
    B: np.ndarray       # (naux, n, n), symmetric in the last two indices
    C: np.ndarray       # (n, n) column-major
    eps: np.ndarray     # (n,)
    H: np.ndarray       # (n, n)
    sigma: float

    @property
    def nvir(self) -> int:
        return self.nbf - self.nocc

    def ao_eri(self) -> np.ndarray:
        """(mu nu|lambda sigma) as an n^4 column-major array (Julia layout)."""
        n = self.nbf
        Bm = self.B.reshape(self.naux, n * n)
        g = Bm.T @ Bm                       # symmetric n^2 x n^2 (C order)
        # g.T is the same matrix as an F-ordered view, so no copy is made at nbf = 200
        return g.T.reshape(n, n, n, n, order="F")

    def wfn(self, ao_eri: Optional[np.ndarray] = None) -> Wfn:
        g = self.ao_eri() if ao_eri is None else ao_eri
        return wfn_from_rhf(self.C, self.eps, g, self.nocc, hao=self.H)


def make_system(nbf: int, nocc: int, naux: int, seed: int = 0,
                sigma: Optional[float] = None) -> SyntheticSystem:
    if not (0 < nocc < nbf):
        raise ValueError("need 0 < nocc < nbf")
    if sigma is None:
        sigma = DEFAULT_B_SCALE / np.sqrt(naux)
    rng = np.random.default_rng(seed)
    n = nbf
    iu = np.triu_indices(n)
    x = rng.normal(0.0, sigma, size=(naux, len(iu[0])))
    B = np.zeros((naux, n, n))
    B[:, iu[0], iu[1]] = x
    B[:, iu[1], iu[0]] = x
    G = rng.normal(0.0, 1.0, size=(n, n))
    C, _ = np.linalg.qr(G)
    eo = np.sort(rng.uniform(-2.0, -0.5, nocc))
    ev = np.sort(rng.uniform(0.2, 3.0, n - nocc))
    X = rng.normal(0.0, 0.5, size=(n, n))
    H = (X + X.T) / np.sqrt(2.0)
    return SyntheticSystem(nbf=n, nocc=nocc, naux=naux, B=B,
                           C=np.asfortranarray(C), eps=np.concatenate([eo, ev]),
                           H=np.asfortranarray(H), sigma=float(sigma))


def make_named(name: str, seed: int = 0, sigma: Optional[float] = None) -> SyntheticSystem:
    n, o, naux = SHAPES[name]
    return make_system(n, o, naux, seed=seed, sigma=sigma)


def batch_specs(count: int = 512, seed: int = 0, nmin: int = 10, nmax: int = 60):
    """Per-system (nbf, nocc, naux, subseed) for the batched workload.

    nbf ~ U{nmin..nmax}, nocc = round(nbf/5), naux = 3*nbf; sub-seeds come from
    ``SeedSequence(seed).spawn(count)``.
    """
    ss = np.random.SeedSequence(seed)
    kids = ss.spawn(count)
    rng = np.random.default_rng(seed)
    nbfs = rng.integers(nmin, nmax + 1, size=count)
    out = []
    for k, n in enumerate(nbfs):
        n = int(n)
        o = max(1, int(round(n / 5)))
        sub = int(kids[k].generate_state(1)[0])
        out.append((n, o, 3 * n, sub))
    return out
