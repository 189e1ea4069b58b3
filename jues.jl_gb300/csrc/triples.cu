// Closed-shell (T) energy correction (src/CoupledCluster/PerturbativeTriples.jl:35-138).
//
// The reference loops over occupied triples i >= j >= k and builds W[a,b,c] (v^3) from twelve
// small contractions per triple.  Here the innermost occupied index rides along in the GEMM
// instead: for each pair (i, j) with j <= i, twelve GETTs write W[a,b,c,k] for every k <= j at
// once (N or M grows by the factor j+1), each reading the reference's operand slices through
// strided modes, so nothing is permuted or copied.  A fused kernel then forms V = W + the
// three (vo|vo) T1 terms on the fly and sums the reference's weighted energy expression over
// a >= b >= c (:117-131).  Partial sums go to fixed per-block slots that are added in a fixed
// order, so the result is deterministic.
#include <algorithm>
#include <vector>

#include "triples.cuh"

namespace jues {

namespace {

constexpr int PT_THREADS = 256;
constexpr int PT_BLOCKS = 152 * 8;

__device__ __forceinline__ double pt_warp_sum(double x) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) x += __shfl_down_sync(0xffffffffu, x, d);
    return x;
}

// W is v x v x v x nk (column-major, k = 0..nk-1 the third occupied index of the pair (i, j)).
// Thread work item t covers one (a >= b >= c) triple (packed a | b << 10 | c << 20) of one k.
__global__ void __launch_bounds__(PT_THREADS) pt_energy_kernel(const double *__restrict__ W, int nk, int i, int j,
                                                               const double *__restrict__ T1, View4 Vvovo,
                                                               const double *__restrict__ fo,
                                                               const double *__restrict__ fv, int o, int v,
                                                               const unsigned *__restrict__ tri, long long ntri,
                                                               double *slots) {
    const long long v2 = (long long)v * v, v3 = v2 * v;
    const long long total = ntri * nk;
    const long long *S = Vvovo.s;
    double acc = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t / ntri);
        const unsigned pk = tri[t % ntri];
        const int a = pk & 1023, b = (pk >> 10) & 1023, c = pk >> 20;
        const double *Wk = W + k * v3;
        auto w = [&](int p, int q, int r) { return Wk[p + (long long)v * q + v2 * r]; };
        // V[p,q,r] = W[p,q,r] + Vvovo[q,j,r,k] T1[i,p] + Vvovo[p,i,r,k] T1[j,q] + Vvovo[p,i,q,j] T1[k,r]  (:113)
        auto vo = [&](int p, int x, int q, int y) { return Vvovo.p[p * S[0] + x * S[1] + q * S[2] + y * S[3]]; };
        auto V = [&](int p, int q, int r, double wpqr) {
            return wpqr + vo(q, j, r, k) * T1[i + (long long)o * p] + vo(p, i, r, k) * T1[j + (long long)o * q] +
                   vo(p, i, q, j) * T1[k + (long long)o * r];
        };
        const double wabc = w(a, b, c), wacb = w(a, c, b), wbac = w(b, a, c);
        const double wbca = w(b, c, a), wcab = w(c, a, b), wcba = w(c, b, a);
        const double vabc = V(a, b, c, wabc), vacb = V(a, c, b, wacb), vbac = V(b, a, c, wbac);
        const double vbca = V(b, c, a, wbca), vcab = V(c, a, b, wcab), vcba = V(c, b, a, wcba);
        const double X = wabc * vabc + wacb * vacb + wbac * vbac + wbca * vbca + wcab * vcab + wcba * vcba;
        const double Y = vabc + vbca + vcab;
        const double Z = vacb + vbac + vcba;
        const double E = (Y - 2.0 * Z) * (wabc + wbca + wcab) + (Z - 2.0 * Y) * (wacb + wbac + wcba) + 3.0 * X;
        const double Dd = fo[i] + fo[j] + fo[k] - fv[a] - fv[b] - fv[c];
        const double num = 2.0 - (i == j) - (j == k);
        const double den = Dd * (1.0 + (a == b) + (b == c));
        acc += E * num / den;
    }
    __shared__ double sh[PT_THREADS / 32];
    acc = pt_warp_sum(acc);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double x = threadIdx.x < PT_THREADS / 32 ? sh[threadIdx.x] : 0.0;
        x = pt_warp_sum(x);
        if (threadIdx.x == 0) slots[blockIdx.x] += x;   // one block per slot, launches in stream order
    }
}

__global__ void pt_sum_slots(const double *slots, int n, double *out) {
    __shared__ double sh[32];
    double x = 0.0;
    for (int s = threadIdx.x; s < n; s += blockDim.x) x += slots[s];
    x = pt_warp_sum(x);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        x = threadIdx.x < (int)(blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        x = pt_warp_sum(x);
        if (threadIdx.x == 0) *out = x;
    }
}

__global__ void pt_zero(double *p, int n) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) p[s] = 0.0;
}

// one W term: W[(rows),(cols)] (+)= alpha sum_x A[(rows),x] B[x,(cols)]
// A operands that are the same slice for every pair sharing i (or j) are kept packed
// (a_const) and dropped at the end
void term(Ctx *ctx, int prec, long long M, long long N, long long K, double alpha, const double *A, Mode mA, Mode kA,
          const double *B, Mode kB, Mode nB, double beta, double *W, Mode mC, Mode nC, const char *name,
          bool a_const = false) {
    GettArgs g;
    g.M = M; g.N = N; g.K = K;
    g.alpha = alpha; g.beta = beta;
    g.A = A; g.mA = mA; g.kA = kA;
    g.B = B; g.kB = kB; g.nB = nB;
    g.C = W; g.mC = mC; g.nC = nC;
    g.a_const = a_const;
    gett(ctx, prec, g, name);
}

}  // namespace

double pT_flops(int o, int v) {
    const double tr = (double)o * (o + 1) * (o + 2) / 6.0;
    return tr * 12.0 * (double)v * v * v * (double)(v + o);
}

double pT_energy(Ctx *ctx, int prec, const double *T1, const double *T2, const View4 &Vv, const View4 &Vo,
                 const View4 &Vvovo, const double *fo, const double *fv, int o, int v) {
    JUES_REQUIRE(o > 0 && v > 0, "need o > 0 and v > 0");
    JUES_REQUIRE(v < 1024, "the (T) energy kernel packs virtual indices in 10 bits (v < 1024)");
    const long long oo = (long long)o * o, oov = oo * v;
    const long long v2 = (long long)v * v, v3 = v2 * v;
    // (a >= b >= c) triples, packed
    std::vector<unsigned> htri;
    htri.reserve((size_t)v * (v + 1) * (v + 2) / 6);
    for (int a = 0; a < v; ++a)
        for (int b = 0; b <= a; ++b)
            for (int c = 0; c <= b; ++c) htri.push_back((unsigned)a | ((unsigned)b << 10) | ((unsigned)c << 20));
    const long long ntri = (long long)htri.size();
    DBuf<unsigned> tri(ctx, htri.size());
    JUES_CHECK_CUDA(cudaMemcpyAsync(tri.p, htri.data(), htri.size() * sizeof(unsigned), cudaMemcpyHostToDevice,
                                    ctx->stream));
    DBuf<double> slots(ctx, PT_BLOCKS + 1);
    pt_zero<<<4, 256, 0, ctx->stream>>>(slots.p, PT_BLOCKS + 1);
    JUES_CHECK_CUDA(cudaGetLastError());
    DBuf<double> W(ctx, (size_t)(v3 * o));   // k = 0..j, at most o of them
    const long long *V0 = Vv.s, *O0 = Vo.s;
    for (int i = 0; i < o; ++i) {
        for (int j = 0; j <= i; ++j) {
            const long long nk = j + 1;
            double *w = W.p;
            const double *Vi = Vv.p + i * V0[3], *Vj = Vv.p + j * V0[3];
            // output modes of the five index groupings of W[a,b,c,k]
            const Mode ab = mode2(v, 1, v), ck = mode2(v, v2, v3);
            const Mode ac = mode2(v, 1, v2), bk = mode2(v, v, v3);
            const Mode ack = mode3(v, v, 1, v2, v3), bck = mode3(v, v, v, v2, v3);
            const Mode bc = mode2(v, v, v2), ak = mode2(v, 1, v3);
            // PerturbativeTriples.jl:104-111; each line below is one term (ijk, ikj, kij, kji, jki, jik)
            // Vvvvo[b,d,a,i] T2[k,j,c,d] -> rows (a,b), cols (c,k)
            term(ctx, prec, v2, v * nk, v, 1.0, Vi, mode2(v, V0[2], V0[0]), plain(V0[1]), T2 + (long long)o * j,
                 plain(oov), mode2(v, oo, 1), 0.0, w, ab, ck, "pt_w", true);
            // - Vvooo[c,k,j,l] T2[i,l,a,b] -> rows (a,b), cols (c,k)
            term(ctx, prec, v2, v * nk, o, -1.0, T2 + i, mode2(v, oo, oov), plain(o), Vo.p + j * O0[2],
                 plain(O0[3]), mode2(v, O0[0], O0[1]), 1.0, w, ab, ck, "pt_w", true);
            // Vvvvo[c,d,a,i] T2[j,k,b,d] -> rows (a,c), cols (b,k)
            term(ctx, prec, v2, v * nk, v, 1.0, Vi, mode2(v, V0[2], V0[0]), plain(V0[1]), T2 + j, plain(oov),
                 mode2(v, oo, o), 1.0, w, ac, bk, "pt_w", true);
            // - Vvooo[b,j,k,l] T2[i,l,a,c] -> rows (a,c), cols (b,k)
            term(ctx, prec, v2, v * nk, o, -1.0, T2 + i, mode2(v, oo, oov), plain(o), Vo.p + j * O0[1],
                 plain(O0[3]), mode2(v, O0[0], O0[2]), 1.0, w, ac, bk, "pt_w", true);
            // Vvvvo[a,d,c,k] T2[j,i,b,d] -> rows (a,c,k), cols b
            term(ctx, prec, v2 * nk, v, v, 1.0, Vv.p, mode3(v, v, V0[0], V0[2], V0[3]), plain(V0[1]),
                 T2 + j + (long long)o * i, plain(oov), plain(oo), 1.0, w, ack, plain(v), "pt_w");
            // - Vvooo[b,j,i,l] T2[k,l,c,a] -> rows (a,c,k), cols b
            term(ctx, prec, v2 * nk, v, o, -1.0, T2, mode3(v, v, oov, oo, 1), plain(o), Vo.p + j * O0[1] + i * O0[2],
                 plain(O0[3]), plain(O0[0]), 1.0, w, ack, plain(v), "pt_w");
            // Vvvvo[b,d,c,k] T2[i,j,a,d] -> rows (b,c,k), cols a
            term(ctx, prec, v2 * nk, v, v, 1.0, Vv.p, mode3(v, v, V0[0], V0[2], V0[3]), plain(V0[1]),
                 T2 + i + (long long)o * j, plain(oov), plain(oo), 1.0, w, bck, plain(1), "pt_w");
            // - Vvooo[a,i,j,l] T2[k,l,c,b] -> rows (b,c,k), cols a
            term(ctx, prec, v2 * nk, v, o, -1.0, T2, mode3(v, v, oov, oo, 1), plain(o), Vo.p + i * O0[1] + j * O0[2],
                 plain(O0[3]), plain(O0[0]), 1.0, w, bck, plain(1), "pt_w");
            // Vvvvo[c,d,b,j] T2[i,k,a,d] -> rows (b,c), cols (a,k)
            term(ctx, prec, v2, v * nk, v, 1.0, Vj, mode2(v, V0[2], V0[0]), plain(V0[1]), T2 + i, plain(oov),
                 mode2(v, oo, o), 1.0, w, bc, ak, "pt_w", true);
            // - Vvooo[a,i,k,l] T2[j,l,b,c] -> rows (b,c), cols (a,k)
            term(ctx, prec, v2, v * nk, o, -1.0, T2 + j, mode2(v, oo, oov), plain(o), Vo.p + i * O0[1],
                 plain(O0[3]), mode2(v, O0[0], O0[2]), 1.0, w, bc, ak, "pt_w", true);
            // Vvvvo[a,d,b,j] T2[k,i,c,d] -> rows (a,b), cols (c,k)
            term(ctx, prec, v2, v * nk, v, 1.0, Vj, mode2(v, V0[0], V0[2]), plain(V0[1]), T2 + (long long)o * i,
                 plain(oov), mode2(v, oo, 1), 1.0, w, ab, ck, "pt_w", true);
            // - Vvooo[c,k,i,l] T2[j,l,b,a] -> rows (a,b), cols (c,k)
            term(ctx, prec, v2, v * nk, o, -1.0, T2 + j, mode2(v, oov, oo), plain(o), Vo.p + i * O0[2],
                 plain(O0[3]), mode2(v, O0[0], O0[1]), 1.0, w, ab, ck, "pt_w", true);
            {
                Ctx::Scope s(ctx, "pt_energy");
                const long long work = ntri * nk;
                const unsigned grid = (unsigned)std::min<long long>((work + PT_THREADS - 1) / PT_THREADS, PT_BLOCKS);
                pt_energy_kernel<<<grid, PT_THREADS, 0, ctx->stream>>>(W.p, (int)nk, i, j, T1, Vvovo, fo, fv, o, v,
                                                                       tri.p, ntri, slots.p);
                JUES_CHECK_CUDA(cudaGetLastError());
            }
        }
    }
    for (int i = 0; i < o; ++i) {   // the kept slices
        pack_cache_drop(ctx, Vv.p + i * V0[3]);
        pack_cache_drop(ctx, T2 + i);
    }
    pt_sum_slots<<<1, 1024, 0, ctx->stream>>>(slots.p, PT_BLOCKS, slots.p + PT_BLOCKS);
    JUES_CHECK_CUDA(cudaGetLastError());
    double et = 0.0;
    JUES_CHECK_CUDA(cudaMemcpyAsync(&et, slots.p + PT_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    JUES_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->check_flags();
    return et;
}

}  // namespace jues
