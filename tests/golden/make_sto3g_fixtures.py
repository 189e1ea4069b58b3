"""Generate the STO-3G fixtures that pin the oracle to the reference's known answers.

The reference's tests quote energies for H2O/STO-3G (``test/TestMollerPlesset.jl:35``:
RMP2 -0.04914964480386458; ``test/TestCoupledCluster.jl:41-45``: RCCD
-0.07015050066089029, RCCSD -0.070680102078571) and three AO integrals of H2/STO-3G
(``test/TestWavefunction.jl:33-35``).  Those came from psi4; psi4 is not installed, so
this script computes the same inputs from first principles:

* STO-3G contractions for H and O (Hehre, Stewart & Pople, J. Chem. Phys. 51, 2657
  (1969), as tabulated in the Basis Set Exchange), contracted functions normalised;
* one- and two-electron integrals by the McMurchie-Davidson Hermite-Gaussian scheme
  (J. Comput. Phys. 26, 218 (1978)) with the Boys function from scipy;
* a tightly converged closed-shell SCF (DIIS on the FPS-SPF commutator).

Geometries are the reference tests' Z-matrices: H2O "O; H 1 1.1; H 1 1.1 2 104.0"
and H2 "H; H 1 1.0", in Angstrom, 1 bohr = 0.52917721067 Angstrom (CODATA 2014, the
value psi4 uses).  Output: ``h2o_sto3g.npz`` (ao_eri, C, eps, nocc) and
``h2_sto3g.npz`` (ao_eri), written next to this file.  Run: ``python
tests/golden/make_sto3g_fixtures.py``.  Test infrastructure only.
"""
import itertools
import math
import os
from functools import lru_cache

import numpy as np
from scipy.special import hyp1f1

BOHR = 0.52917721067
STO3G_COEF_1S = (0.15432897, 0.53532814, 0.44463454)
STO3G = {
    "H": [(0, (3.42525091, 0.62391373, 0.16885540), STO3G_COEF_1S)],
    "O": [(0, (130.7093200, 23.8088610, 6.4436083), STO3G_COEF_1S),
          (0, (5.0331513, 1.1695961, 0.3803890), (-0.09996723, 0.39951283, 0.70011547)),
          (1, (5.0331513, 1.1695961, 0.3803890), (0.15591627, 0.60768372, 0.39195739))],
}
ZNUC = {"H": 1.0, "O": 8.0}


def boys(m, T):
    return hyp1f1(m + 0.5, m + 1.5, -T) / (2.0 * m + 1.0)


def dfact(n):
    return 1.0 if n <= 0 else float(np.prod(np.arange(n, 0, -2)))


class CGTO:
    def __init__(self, center, lmn, exps, coefs):
        self.A = np.asarray(center, float)
        self.lmn = lmn
        self.exps = np.asarray(exps, float)
        L = sum(lmn)
        pre = [(2 * a / math.pi) ** 0.75 * (4 * a) ** (L / 2)
               / math.sqrt(dfact(2 * lmn[0] - 1) * dfact(2 * lmn[1] - 1) * dfact(2 * lmn[2] - 1))
               for a in self.exps]
        self.c = np.asarray(coefs, float) * np.asarray(pre)
        s = 0.0                       # normalise the contraction
        for (ca, a), (cb, b) in itertools.product(zip(self.c, self.exps), repeat=2):
            s += ca * cb * overlap_prim(a, lmn, self.A, b, lmn, self.A)
        self.c /= math.sqrt(s)


def E(i, j, t, Qx, a, b):
    p = a + b
    q = a * b / p
    if t < 0 or t > i + j:
        return 0.0
    if i == j == t == 0:
        return math.exp(-q * Qx * Qx)
    if j == 0:
        return (E(i - 1, j, t - 1, Qx, a, b) / (2 * p) - q * Qx / a * E(i - 1, j, t, Qx, a, b)
                + (t + 1) * E(i - 1, j, t + 1, Qx, a, b))
    return (E(i, j - 1, t - 1, Qx, a, b) / (2 * p) + q * Qx / b * E(i, j - 1, t, Qx, a, b)
            + (t + 1) * E(i, j - 1, t + 1, Qx, a, b))


def overlap_prim(a, lmn1, A, b, lmn2, B):
    s = 1.0
    for d in range(3):
        s *= E(lmn1[d], lmn2[d], 0, A[d] - B[d], a, b)
    return s * (math.pi / (a + b)) ** 1.5


def kinetic_prim(a, lmn1, A, b, lmn2, B):
    l, m, n = lmn2
    t0 = b * (2 * (l + m + n) + 3) * overlap_prim(a, lmn1, A, b, lmn2, B)
    t1 = -2 * b * b * (overlap_prim(a, lmn1, A, b, (l + 2, m, n), B)
                       + overlap_prim(a, lmn1, A, b, (l, m + 2, n), B)
                       + overlap_prim(a, lmn1, A, b, (l, m, n + 2), B))
    t2 = -0.5 * (l * (l - 1) * overlap_prim(a, lmn1, A, b, (l - 2, m, n), B) if l > 1 else 0.0)
    t2 += -0.5 * (m * (m - 1) * overlap_prim(a, lmn1, A, b, (l, m - 2, n), B) if m > 1 else 0.0)
    t2 += -0.5 * (n * (n - 1) * overlap_prim(a, lmn1, A, b, (l, m, n - 2), B) if n > 1 else 0.0)
    return t0 + t1 + t2


def R(t, u, v, n, p, PCx, PCy, PCz, RPC):
    @lru_cache(maxsize=None)
    def r(t, u, v, n):
        if t < 0 or u < 0 or v < 0:
            return 0.0
        if t == u == v == 0:
            return (-2 * p) ** n * boys(n, p * RPC * RPC)
        if t == u == 0:
            return (v - 1) * r(t, u, v - 2, n + 1) + PCz * r(t, u, v - 1, n + 1)
        if t == 0:
            return (u - 1) * r(t, u - 2, v, n + 1) + PCy * r(t, u - 1, v, n + 1)
        return (t - 1) * r(t - 2, u, v, n + 1) + PCx * r(t - 1, u, v, n + 1)
    return r(t, u, v, n)


def nuclear_prim(a, lmn1, A, b, lmn2, B, C):
    p = a + b
    P = (a * A + b * B) / p
    PC = P - C
    RPC = np.linalg.norm(PC)
    l1, m1, n1 = lmn1
    l2, m2, n2 = lmn2
    s = 0.0
    for t in range(l1 + l2 + 1):
        for u in range(m1 + m2 + 1):
            for v in range(n1 + n2 + 1):
                s += (E(l1, l2, t, A[0] - B[0], a, b) * E(m1, m2, u, A[1] - B[1], a, b)
                      * E(n1, n2, v, A[2] - B[2], a, b) * R(t, u, v, 0, p, *PC, RPC))
    return 2 * math.pi / p * s


def eri_prim(a, lmn1, A, b, lmn2, B, c, lmn3, C, d, lmn4, D):
    p = a + b
    q = c + d
    alpha = p * q / (p + q)
    P = (a * A + b * B) / p
    Q = (c * C + d * D) / q
    PQ = P - Q
    RPQ = np.linalg.norm(PQ)

    @lru_cache(maxsize=None)
    def r(t, u, v, n):
        if t < 0 or u < 0 or v < 0:
            return 0.0
        if t == u == v == 0:
            return (-2 * alpha) ** n * boys(n, alpha * RPQ * RPQ)
        if t == u == 0:
            return (v - 1) * r(t, u, v - 2, n + 1) + PQ[2] * r(t, u, v - 1, n + 1)
        if t == 0:
            return (u - 1) * r(t, u - 2, v, n + 1) + PQ[1] * r(t, u - 1, v, n + 1)
        return (t - 1) * r(t - 2, u, v, n + 1) + PQ[0] * r(t - 1, u, v, n + 1)

    Eab = [[E(lmn1[k], lmn2[k], t, A[k] - B[k], a, b) for t in range(lmn1[k] + lmn2[k] + 1)]
           for k in range(3)]
    Ecd = [[E(lmn3[k], lmn4[k], t, C[k] - D[k], c, d) for t in range(lmn3[k] + lmn4[k] + 1)]
           for k in range(3)]
    s = 0.0
    for t, et in enumerate(Eab[0]):
        for u, eu in enumerate(Eab[1]):
            for v, ev in enumerate(Eab[2]):
                e1 = et * eu * ev
                if e1 == 0.0:
                    continue
                for tau, f in enumerate(Ecd[0]):
                    for nu, g in enumerate(Ecd[1]):
                        for phi, h in enumerate(Ecd[2]):
                            s += (e1 * f * g * h * (-1) ** (tau + nu + phi)
                                  * r(t + tau, u + nu, v + phi, 0))
    return 2 * math.pi ** 2.5 / (p * q * math.sqrt(p + q)) * s


def build_basis(atoms):
    bas = []
    for sym, xyz in atoms:
        for L, exps, coefs in STO3G[sym]:
            lmns = [(0, 0, 0)] if L == 0 else [(1, 0, 0), (0, 1, 0), (0, 0, 1)]
            for lmn in lmns:
                bas.append(CGTO(xyz, lmn, exps, coefs))
    return bas


def contract(f, g1, g2):
    return sum(ca * cb * f(a, g1.lmn, g1.A, b, g2.lmn, g2.A)
               for ca, a in zip(g1.c, g1.exps) for cb, b in zip(g2.c, g2.exps))


def integrals(atoms):
    bas = build_basis(atoms)
    n = len(bas)
    S = np.zeros((n, n))
    T = np.zeros((n, n))
    V = np.zeros((n, n))
    for i, j in itertools.product(range(n), repeat=2):
        S[i, j] = contract(overlap_prim, bas[i], bas[j])
        T[i, j] = contract(kinetic_prim, bas[i], bas[j])
        for sym, xyz in atoms:
            C = np.asarray(xyz, float)
            V[i, j] -= ZNUC[sym] * contract(
                lambda a, l1, A, b, l2, B: nuclear_prim(a, l1, A, b, l2, B, C), bas[i], bas[j])
    g = np.zeros((n, n, n, n))
    done = {}
    for i, j, k, l in itertools.product(range(n), repeat=4):
        key = tuple(sorted([tuple(sorted((i, j))), tuple(sorted((k, l)))]))
        if key not in done:
            gi, gj, gk, gl = bas[i], bas[j], bas[k], bas[l]
            s = 0.0
            for ca, a in zip(gi.c, gi.exps):
                for cb, b in zip(gj.c, gj.exps):
                    for cc, c in zip(gk.c, gk.exps):
                        for cd, d in zip(gl.c, gl.exps):
                            s += ca * cb * cc * cd * eri_prim(a, gi.lmn, gi.A, b, gj.lmn, gj.A,
                                                              c, gk.lmn, gk.A, d, gl.lmn, gl.A)
            done[key] = s
        g[i, j, k, l] = done[key]
    return S, T + V, g


def rhf(S, H, g, nocc, maxit=200, tol=1e-13):
    s, U = np.linalg.eigh(S)
    X = U @ np.diag(s ** -0.5) @ U.T
    e0, C0 = np.linalg.eigh(X.T @ H @ X)          # core-Hamiltonian guess
    C0 = X @ C0
    Dm = C0[:, :nocc] @ C0[:, :nocc].T
    fs, es = [], []
    for it in range(maxit):
        J = np.einsum("pqrs,rs->pq", g, Dm)
        K = np.einsum("prqs,rs->pq", g, Dm)
        F = H + 2 * J - K
        err = X.T @ (F @ Dm @ S - S @ Dm @ F) @ X
        fs.append(F)
        es.append(err)
        if len(fs) > 8:
            fs.pop(0)
            es.pop(0)
        if it > 1:
            m = len(fs)
            B = -np.ones((m + 1, m + 1))
            B[m, m] = 0
            for a in range(m):
                for b in range(m):
                    B[a, b] = np.sum(es[a] * es[b])
            rhs = np.zeros(m + 1)
            rhs[m] = -1
            c = np.linalg.lstsq(B, rhs, rcond=None)[0]
            F = sum(c[k] * fs[k] for k in range(m))
        eps, Cp = np.linalg.eigh(X.T @ F @ X)
        C = X @ Cp
        Dn = C[:, :nocc] @ C[:, :nocc].T
        if np.abs(Dn - Dm).max() < tol and np.abs(err).max() < tol:
            Dm = Dn
            break
        Dm = Dn
    J = np.einsum("pqrs,rs->pq", g, Dm)
    K = np.einsum("prqs,rs->pq", g, Dm)
    F = H + 2 * J - K
    eps, Cp = np.linalg.eigh(X.T @ F @ X)
    return X @ Cp, eps


def zmat_h2o(r=1.1, theta=104.0):
    r /= BOHR
    th = math.radians(theta)
    return [("O", (0.0, 0.0, 0.0)), ("H", (0.0, 0.0, r)),
            ("H", (r * math.sin(th), 0.0, r * math.cos(th)))]


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    atoms = zmat_h2o()
    S, H, g = integrals(atoms)
    C, eps = rhf(S, H, g, 5)
    np.savez(os.path.join(here, "h2o_sto3g.npz"), ao_eri=g, C=C, eps=eps, nocc=5,
             S=S, H=H)
    h2 = [("H", (0.0, 0.0, 0.0)), ("H", (0.0, 0.0, 1.0 / BOHR))]
    _, _, g2 = integrals(h2)
    np.savez(os.path.join(here, "h2_sto3g.npz"), ao_eri=g2)
    print("written", eps)


if __name__ == "__main__":
    main()
