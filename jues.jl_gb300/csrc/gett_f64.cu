// FP64 tensor contraction as a GEMM over composite tensor modes (the plain, drop-in form).
//
// GB300 executes FP64 on its CUDA cores only (there is no FP64 kind for tcgen05), so this
// kernel is DFMA-issue bound: BM x BN output tiles, (BM/16) x (BN/16) register blocking per
// thread, operand tiles staged in shared memory with the per-row / per-column element offsets
// of the composite modes precomputed once per tile.  The same tile routine serves single
// problems and the grouped (batched) form, whose persistent CTAs walk a tile list that spans
// many independent problems.
#include <algorithm>
#include <string>

#include "common.cuh"
#include "convert.cuh"
#include "gett_f64.cuh"

namespace jues {

namespace {

constexpr int BK = 16, NT = 256;

template <int BM, int BN>
struct TileSmem {
    double As[BK][BM + 1];
    double Bs[BK][BN + 1];
    long long offA[BM], offB[BN], offCm[BM], offCn[BN];
    long long koA[BK], koB[BK];
};

template <int BM, int BN>
__device__ __forceinline__ void gett_tile(const GroupProblem &g, long long tile, TileSmem<BM, BN> &sm,
                                          long long kbeg, long long kend) {
    constexpr int TM = BM / 16, TN = BN / 16;
    const int tid = threadIdx.x;
    const long long m0 = (tile % g.mtiles) * BM;
    const long long n0 = (tile / g.mtiles) * BN;
    const int a_mfast = (g.mA.s0 == 1 && g.mA.d0 > 1);
    const int b_nfast = (g.nB.s0 == 1 && g.nB.d0 > 1);
    const int c_mfast = (g.mC.s0 == 1 && g.mC.d0 > 1);
    __syncthreads();   // the previous tile of a persistent CTA is done with the tables
    for (int r = tid; r < BM; r += NT) {
        const long long m = m0 + r;
        sm.offA[r] = m < g.M ? mode_off(g.mA, m) : -1;
        sm.offCm[r] = m < g.M ? mode_off(g.mC, m) : -1;
    }
    for (int c = tid; c < BN; c += NT) {
        const long long n = n0 + c;
        sm.offB[c] = n < g.N ? mode_off(g.nB, n) : -1;
        sm.offCn[c] = n < g.N ? mode_off(g.nC, n) : -1;
    }
    const int tr = c_mfast ? (tid & 15) : (tid >> 4);
    const int tc = c_mfast ? (tid >> 4) : (tid & 15);
    double acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = 0.0;

    for (long long k0 = kbeg; k0 < kend; k0 += BK) {
        __syncthreads();
        if (tid < BK) {
            const long long k = k0 + tid;
            sm.koA[tid] = k < kend ? mode_off(g.kA, k) : -1;
        } else if (tid >= 32 && tid < 32 + BK) {
            const long long k = k0 + tid - 32;
            sm.koB[tid - 32] = k < kend ? mode_off(g.kB, k) : -1;
        }
        __syncthreads();
        for (int e = tid; e < BM * BK; e += NT) {
            const int m = a_mfast ? (e % BM) : (e / BK);
            const int k = a_mfast ? (e / BM) : (e % BK);
            const long long om = sm.offA[m], ok = sm.koA[k];
            sm.As[k][m] = (om >= 0 && ok >= 0) ? __ldg(g.A + om + ok) : 0.0;
        }
        for (int e = tid; e < BN * BK; e += NT) {
            const int n = b_nfast ? (e % BN) : (e / BK);
            const int k = b_nfast ? (e / BN) : (e % BK);
            const long long on = sm.offB[n], ok = sm.koB[k];
            sm.Bs[k][n] = (on >= 0 && ok >= 0) ? __ldg(g.B + on + ok) : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double a[TM], b[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) a[i] = sm.As[kk][tr + 16 * i];
#pragma unroll
            for (int j = 0; j < TN; ++j) b[j] = sm.Bs[kk][tc + 16 * j];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        const long long om = sm.offCm[tr + 16 * i];
        if (om < 0) continue;
        // a row's inputs are loaded before any of its outputs is stored (each element is this
        // thread's alone; C and Cin may alias), so those loads are in flight together
        double cin[TN];
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const long long on = sm.offCn[tc + 16 * j];
            cin[j] = (g.beta != 0.0 && on >= 0) ? g.Cin[om + on] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const long long on = sm.offCn[tc + 16 * j];
            if (on < 0) continue;
            double v = g.alpha * acc[i][j];
            if (g.beta != 0.0) v = fma(g.beta, cin[j], v);
            g.C[om + on] = v;
        }
    }
}

template <int BM, int BN>
__global__ void __launch_bounds__(NT) gett_f64_kernel(GroupProblem g) {
    __shared__ TileSmem<BM, BN> sm;
    gett_tile<BM, BN>(g, blockIdx.x, sm, 0, g.K);
}

// split-K form: CTA b contracts K range [s kper, min(K, (s+1) kper)), s = b / tiles, of tile
// b % tiles into the plain column-major partial ws[s] (M x N; g's output modes describe it)
template <int BM, int BN>
__global__ void __launch_bounds__(NT) gett_f64_splitk(GroupProblem g, long long tiles, long long kper) {
    __shared__ TileSmem<BM, BN> sm;
    const long long s = blockIdx.x / tiles;
    g.C += s * g.M * g.N;
    g.Cin = g.C;
    gett_tile<BM, BN>(g, blockIdx.x % tiles, sm, s * kper, min(g.K, (s + 1) * kper));
}

template <class T>
__global__ void splitk_reduce_kernel(const T *__restrict__ ws, int ks, long long sstride, long long ld, long long M,
                                     long long N, double alpha, double beta, double *C, const double *Cin, Mode mC,
                                     Mode nC) {
    // GB300 runs FP64 at about two operations per clock per SM: the FP32 partials convert on the
    // integer pipes, and alpha = 1 and beta = 0 cost nothing
    const long long total = M * N;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        long long m, n;
        divmod_ll(i, M, n, m);
        const T *p = ws + n * ld + m;
        // eight partials loaded ahead of their (in-order) sum, so the loads overlap
        double acc = 0.0;
        int s = 0;
        for (; s + 8 <= ks; s += 8) {
            T v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = p[(long long)(s + u) * sstride];
#pragma unroll
            for (int u = 0; u < 8; ++u) acc += to_f64(v[u]);
        }
        for (; s < ks; ++s) acc += to_f64(p[(long long)s * sstride]);
        const long long off = mode_off(mC, m) + mode_off(nC, n);
        double v = alpha == 1.0 ? acc : alpha * acc;
        if (beta != 0.0) v = fma(beta, Cin[off], v);
        C[off] = v;
    }
}

template <class T>
void splitk_reduce_t(Ctx *ctx, const T *ws, int ks, long long sstride, long long ld, long long M, long long N,
                     double alpha, double beta, double *C, const double *Cin, const Mode &mC, const Mode &nC,
                     const char *name) {
    const long long total = M * N;
    const long long blocks = std::min<long long>((total + 255) / 256, 152LL * 8);
    const std::string nm = std::string(name) + ".reduce";
    Ctx::Scope sc(ctx, nm.c_str());
    splitk_reduce_kernel<T><<<(unsigned)blocks, 256, 0, ctx->stream>>>(ws, ks, sstride, ld, M, N, alpha, beta, C,
                                                                      Cin ? Cin : C, mC, nC);
    JUES_CHECK_CUDA(cudaGetLastError());
}

// persistent grouped form: problem p owns tiles [tile_start[p], tile_start[p+1])
template <int BM, int BN>
__global__ void __launch_bounds__(NT) gett_f64_grouped(const GroupProblem *__restrict__ probs, int nprob,
                                                       long long total) {
    __shared__ TileSmem<BM, BN> sm;
    for (long long t = blockIdx.x; t < total; t += gridDim.x) {
        int lo = 0, hi = nprob - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (probs[mid].tile_start <= t) lo = mid; else hi = mid - 1;
        }
        gett_tile<BM, BN>(probs[lo], t - probs[lo].tile_start, sm, 0, probs[lo].K);
    }
}

// Offset of a mode index that advances by a fixed step: the division-free successor of
// mode_off (the carries replace the divisions), so a K loop costs a few integer adds per
// element instead of 32- or 64-bit divisions.
struct ModeIter {
    int i0, i1;          // the mode's first two sub-indices (unused for a single-stride mode)
    long long off;
    __device__ __forceinline__ void init(const Mode &m, long long r) {
        if (m.d0 == MODE_BIG) {
            i0 = i1 = 0;
            off = r * m.s0;
            return;
        }
        long long q, r0;
        divmod_ll(r, m.d0, q, r0);
        i0 = (int)r0;
        if (m.d1 == MODE_BIG) {
            i1 = 0;
            off = r0 * m.s0 + q * m.s1;
            return;
        }
        long long q2, r1;
        divmod_ll(q, m.d1, q2, r1);
        i1 = (int)r1;
        off = r0 * m.s0 + r1 * m.s1 + q2 * m.s2;
    }
    __device__ __forceinline__ void step(const Mode &m, int by) {
        if (m.d0 == MODE_BIG) {
            off += by * m.s0;
            return;
        }
        i0 += by;
        off += by * m.s0;
        while (i0 >= m.d0) {
            i0 -= (int)m.d0;
            off += m.s1 - m.d0 * m.s0;
            if (m.d1 != MODE_BIG && ++i1 >= m.d1) {
                i1 = 0;
                off += m.s2 - m.d1 * m.s1;
            }
        }
    }
};

// skinny GEMM (N <= NN <= 8): one warp per output row, lanes split K
template <int NN>
__global__ void __launch_bounds__(256, NN == 1 ? 3 : 2) gett_f64_skinny(GroupProblem g) {
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= g.M) return;
    const long long m = warp;
    const long long om = mode_off(g.mA, m);
    double acc[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) acc[j] = 0.0;
    long long onb[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) onb[j] = j < g.N ? mode_off(g.nB, j) : 0;
    // four independent K positions per lane (k, k + 32, k + 64, k + 96): their loads are in
    // flight together instead of one load latency per element
    constexpr int U = 4;
    ModeIter ia[U], ib[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        ia[u].init(g.kA, lane + 32 * u);
        ib[u].init(g.kB, lane + 32 * u);
    }
    for (long long k = lane; k < g.K; k += 32 * U) {
        double a[U];
#pragma unroll
        for (int u = 0; u < U; ++u) a[u] = k + 32 * u < g.K ? __ldg(g.A + om + ia[u].off) : 0.0;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (k + 32 * u < g.K) {
                const long long ok = ib[u].off;
#pragma unroll
                for (int j = 0; j < NN; ++j)
                    if (j < g.N) acc[j] = fma(a[u], __ldg(g.B + ok + onb[j]), acc[j]);
            }
            ia[u].step(g.kA, 32 * U);
            ib[u].step(g.kB, 32 * U);
        }
    }
    const long long oc = mode_off(g.mC, m);
#pragma unroll
    for (int j = 0; j < NN; ++j) {
        if (j >= g.N) break;
        double v = acc[j];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
        if (lane == 0) {
            const long long off = oc + mode_off(g.nC, j);
            double r = g.alpha * v;
            if (g.beta != 0.0) r = fma(g.beta, g.Cin[off], r);
            g.C[off] = r;
        }
    }
}

// skinny GEMM (N <= NN <= 8) whose rows, not K, are the unit-stride index of A: one thread per
// output row, so a warp's loads of one K position are 32 consecutive doubles; blockIdx.y takes
// K positions [y kper, (y + 1) kper) (four independent positions in flight per thread) and writes
// its partial sums to part[y][n][m] for the split-K reduction (kper = K: one part)
template <int NN>
__global__ void __launch_bounds__(256) gett_f64_rows(GroupProblem g, long long kper, double *__restrict__ part) {
    const long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (m >= g.M) return;
    const long long k0 = blockIdx.y * kper, k1 = min(g.K, k0 + kper);
    const long long om = mode_off(g.mA, m);
    long long onb[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) onb[j] = j < g.N ? mode_off(g.nB, j) : 0;
    double acc[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) acc[j] = 0.0;
    constexpr int U = 4;
    ModeIter ia[U], ib[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        ia[u].init(g.kA, k0 + u);
        ib[u].init(g.kB, k0 + u);
    }
    for (long long k = k0; k < k1; k += U) {
        double a[U];
#pragma unroll
        for (int u = 0; u < U; ++u) a[u] = k + u < k1 ? __ldg(g.A + om + ia[u].off) : 0.0;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (k + u < k1) {
                const long long ok = ib[u].off;
#pragma unroll
                for (int j = 0; j < NN; ++j)
                    if (j < g.N) acc[j] = fma(a[u], __ldg(g.B + ok + onb[j]), acc[j]);
            }
            ia[u].step(g.kA, U);
            ib[u].step(g.kB, U);
        }
    }
#pragma unroll
    for (int j = 0; j < NN; ++j)
        if (j < g.N) part[(blockIdx.y * g.N + j) * g.M + m] = acc[j];
}

// small GEMM (M N <= 2^16 outputs, K <= 8192): one warp per output element, its lanes over K,
// so that even a single-tile problem spreads over the whole GPU instead of one CTA
__global__ void __launch_bounds__(256) gett_f64_small(GroupProblem g) {
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= g.M * g.N) return;
    const long long m = w % g.M, n = w / g.M;
    const long long oa = mode_off(g.mA, m), ob = mode_off(g.nB, n);
    ModeIter ia, ib;
    ia.init(g.kA, lane);
    ib.init(g.kB, lane);
    double acc = 0.0;
    for (long long k = lane; k < g.K; k += 32) {
        acc = fma(__ldg(g.A + oa + ia.off), __ldg(g.B + ob + ib.off), acc);
        ia.step(g.kA, 32);
        ib.step(g.kB, 32);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, d);
    if (lane == 0) {
        const long long off = mode_off(g.mC, m) + mode_off(g.nC, n);
        double r = g.alpha * acc;
        if (g.beta != 0.0) r = fma(g.beta, g.Cin[off], r);
        g.C[off] = r;
    }
}

}  // namespace

GroupProblem to_problem(const GettArgs &a) {
    GroupProblem g;
    g.M = a.M; g.N = a.N; g.K = a.K;
    g.alpha = a.alpha; g.beta = a.beta;
    g.A = a.A; g.mA = a.mA; g.kA = a.kA;
    g.B = a.B; g.kB = a.kB; g.nB = a.nB;
    g.C = a.C; g.mC = a.mC; g.nC = a.nC;
    g.Cin = a.Cin ? a.Cin : a.C;
    g.mtiles = 1;
    g.tile_start = 0;
    return g;
}

void gett_f64(Ctx *ctx, const GettArgs &a, const char *name) {
    if (a.M <= 0 || a.N <= 0) return;
    GroupProblem g = to_problem(a);
    if (a.N > 8 && a.M * a.N <= (1LL << 16) && a.K <= 8192) {
        Ctx::Scope s(ctx, name);
        gett_f64_small<<<(unsigned)((a.M * a.N * 32 + 255) / 256), 256, 0, ctx->stream>>>(g);
        JUES_CHECK_CUDA(cudaGetLastError());
        return;
    }
    const bool k_unit = a.kA.s0 == 1 && a.kA.d0 > 1, rows_unit = a.mA.s0 == 1 && a.mA.d0 > 1;
    if (a.N <= 8 && rows_unit && !k_unit && a.M >= 256) {
        // thread per row, K split over blockIdx.y so that about eight blocks run per SM
        const long long rb = (a.M + 255) / 256;
        long long ks = std::max<long long>(1, std::min<long long>((152LL * 8 + rb - 1) / rb, a.K / 64));
        ks = std::min<long long>(ks, 65535);
        long long kper = (a.K + ks - 1) / ks;
        kper = (kper + 3) / 4 * 4;
        ks = (a.K + kper - 1) / kper;
        JUES_REQUIRE(rb < (1LL << 31), "GEMM too large for one launch");
        double *ws = static_cast<double *>(ctx->splitk_scratch((size_t)(ks * a.M * a.N) * sizeof(double)));
        {
            Ctx::Scope s(ctx, name);
            const dim3 grid((unsigned)rb, (unsigned)ks);
            if (a.N == 1)
                gett_f64_rows<1><<<grid, 256, 0, ctx->stream>>>(g, kper, ws);
            else
                gett_f64_rows<8><<<grid, 256, 0, ctx->stream>>>(g, kper, ws);
            JUES_CHECK_CUDA(cudaGetLastError());
        }
        splitk_reduce(ctx, ws, (int)ks, a.M * a.N, a.M, a.M, a.N, a.alpha, a.beta, a.C, g.Cin, a.mC, a.nC, name);
        return;
    }
    if (a.N <= 8) {
        long long blocks = (a.M * 32 + 255) / 256;
        JUES_REQUIRE(blocks < (1LL << 31), "GEMM too large for one launch");
        Ctx::Scope s(ctx, name);
        if (a.N == 1)
            gett_f64_skinny<1><<<(unsigned)blocks, 256, 0, ctx->stream>>>(g);
        else
            gett_f64_skinny<8><<<(unsigned)blocks, 256, 0, ctx->stream>>>(g);
        JUES_CHECK_CUDA(cudaGetLastError());
        return;
    }
    g.mtiles = (a.M + 63) / 64;
    const long long tiles = g.mtiles * ((a.N + 63) / 64);
    JUES_REQUIRE(tiles < (1LL << 31), "GEMM too large for one launch");
    // A grid below four CTAs per SM with a long K splits K (at least 512 per split); the
    // partials are reduced in FP64 in split order.
    constexpr long long kTarget = 152LL * 4;
    if (tiles < kTarget && a.K >= 1024) {
        const long long want = std::min<long long>((kTarget + tiles - 1) / tiles, a.K / 512);
        long long kper = (a.K + want - 1) / want;
        kper = (kper + BK - 1) / BK * BK;
        const long long ks = (a.K + kper - 1) / kper;
        if (ks > 1) {
            double *ws = static_cast<double *>(ctx->splitk_scratch((size_t)(ks * a.M * a.N) * sizeof(double)));
            GroupProblem p = g;
            p.C = ws;
            p.Cin = ws;
            p.mC = plain(1);
            p.nC = plain(a.M);
            p.alpha = 1.0;
            p.beta = 0.0;
            {
                Ctx::Scope s(ctx, name);
                gett_f64_splitk<64, 64><<<(unsigned)(tiles * ks), NT, 0, ctx->stream>>>(p, tiles, kper);
                JUES_CHECK_CUDA(cudaGetLastError());
            }
            splitk_reduce(ctx, ws, (int)ks, a.M * a.N, a.M, a.M, a.N, a.alpha, a.beta, a.C, g.Cin, a.mC, a.nC, name);
            return;
        }
    }
    Ctx::Scope s(ctx, name);
    gett_f64_kernel<64, 64><<<(unsigned)tiles, NT, 0, ctx->stream>>>(g);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void splitk_reduce(Ctx *ctx, const float *ws, int ks, long long sstride, long long ld, long long M, long long N,
                   double alpha, double beta, double *C, const double *Cin, const Mode &mC, const Mode &nC,
                   const char *name) {
    splitk_reduce_t(ctx, ws, ks, sstride, ld, M, N, alpha, beta, C, Cin, mC, nC, name);
}
void splitk_reduce(Ctx *ctx, const double *ws, int ks, long long sstride, long long ld, long long M, long long N,
                   double alpha, double beta, double *C, const double *Cin, const Mode &mC, const Mode &nC,
                   const char *name) {
    splitk_reduce_t(ctx, ws, ks, sstride, ld, M, N, alpha, beta, C, Cin, mC, nC, name);
}

const TileShape kTileShapes[kNumTileShapes] = {{64, 64}, {32, 64}, {64, 32}, {32, 32}};

long long grouped_tiles(std::vector<GroupProblem> &probs, int shape) {
    const int BM = kTileShapes[shape].bm, BN = kTileShapes[shape].bn;
    long long start = 0;
    for (auto &p : probs) {
        p.mtiles = (p.M + BM - 1) / BM;
        p.tile_start = start;
        start += (p.M > 0 && p.N > 0) ? p.mtiles * ((p.N + BN - 1) / BN) : 0;
    }
    return start;
}

void gett_f64_grouped_launch(Ctx *ctx, const GroupProblem *d_probs, int nprob, long long total, int shape,
                             const char *name) {
    if (total <= 0) return;
    const long long grid = std::min<long long>(total, 152LL * 4);   // persistent: 4 CTAs per SM
    Ctx::Scope s(ctx, name);
    switch (shape) {
        case 0: gett_f64_grouped<64, 64><<<(unsigned)grid, NT, 0, ctx->stream>>>(d_probs, nprob, total); break;
        case 1: gett_f64_grouped<32, 64><<<(unsigned)grid, NT, 0, ctx->stream>>>(d_probs, nprob, total); break;
        case 2: gett_f64_grouped<64, 32><<<(unsigned)grid, NT, 0, ctx->stream>>>(d_probs, nprob, total); break;
        default: gett_f64_grouped<32, 32><<<(unsigned)grid, NT, 0, ctx->stream>>>(d_probs, nprob, total); break;
    }
    JUES_CHECK_CUDA(cudaGetLastError());
}

void gett(Ctx *ctx, int precision, const GettArgs &g, const char *name) {
    if (precision == JUES_PREC_SPLIT || precision == JUES_PREC_SPLIT2)
        gett_tc(ctx, g, name, 2);
    else if (precision == JUES_PREC_SPLIT3)
        gett_tc(ctx, g, name, 3);
    else
        gett_f64(ctx, g, name);
}

}  // namespace jues
