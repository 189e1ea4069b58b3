// Fock matrix of a closed-shell determinant (src/Backend/IntegralTransformation.jl:119-141):
//     f[p,q] = sum C[mu,p] C[nu,q] (h[mu,nu] + 2 J[mu,nu] - K[mu,nu]),
//     J[mu,nu] = sum_{lam,sig} g[mu,nu,lam,sig] D[lam,sig],  K[mu,nu] = sum g[mu,lam,nu,sig] D[lam,sig],
//     D = Co Co^T.
// J and K are matrix-vector contractions of the AO integrals against D, read through the
// composite modes of the reference's index order (no symmetry of g is assumed), so each is one
// pass over g.  Everything is FP64.
#include "common.cuh"
#include "fock.cuh"

namespace jues {

void get_fock(Ctx *ctx, const double *g, const double *h, int n, const double *C, int nmo, const double *Co, int o,
              double *f) {
    JUES_REQUIRE(n > 0 && nmo > 0 && o >= 0, "bad Fock dimensions");
    const long long nn = (long long)n * n;
    DBuf<double> D(ctx, (size_t)nn), F(ctx, (size_t)nn), tmp(ctx, (size_t)n * nmo);
    auto G = [&](long long M, long long N, long long K, double alpha, const double *A, Mode mA, Mode kA,
                 const double *B, Mode kB, Mode nB, double beta, double *Cm, Mode mC, Mode nC, const char *name) {
        GettArgs a;
        a.M = M; a.N = N; a.K = K;
        a.alpha = alpha; a.beta = beta;
        a.A = A; a.mA = mA; a.kA = kA;
        a.B = B; a.kB = kB; a.nB = nB;
        a.C = Cm; a.mC = mC; a.nC = nC;
        gett_f64(ctx, a, name);
    };
    // D[lam,sig] = sum_k Co[lam,k] Co[sig,k]
    if (o > 0)
        G(n, n, o, 1.0, Co, plain(1), plain(n), Co, plain(n), plain(1), 0.0, D.p, plain(1), plain(n), "fock_density");
    else
        fill(ctx, D.p, (size_t)nn, 0.0);
    // F = h + 2 J - K
    JUES_CHECK_CUDA(cudaMemcpyAsync(F.p, h, (size_t)nn * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    // J: rows (mu,nu) = offset r, contraction (lam,sig) = offset n^2 k
    G(nn, 1, nn, 2.0, g, plain(1), plain(nn), D.p, plain(1), plain(0), 1.0, F.p, plain(1), plain(0), "fock_j");
    // K: rows (mu,nu) -> g offset mu + n^2 nu, contraction (lam,sig) -> n lam + n^3 sig
    G(nn, 1, nn, -1.0, g, mode2(n, 1, nn), mode2(n, n, nn * n), D.p, plain(1), plain(0), 1.0, F.p, plain(1),
      plain(0), "fock_k");
    // f = C^T F C
    G(n, nmo, n, 1.0, F.p, plain(1), plain(n), C, plain(1), plain(n), 0.0, tmp.p, plain(1), plain(n), "fock_mo");
    G(nmo, nmo, n, 1.0, C, plain(n), plain(1), tmp.p, plain(1), plain(n), 0.0, f, plain(1), plain(nmo), "fock_mo");
}

}  // namespace jues
