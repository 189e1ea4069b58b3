// FP64 tensor contraction as a GEMM over composite tensor modes (the plain, drop-in form).
//
// GB300 executes FP64 on its CUDA cores only (there is no FP64 kind for tcgen05), so this
// kernel is DFMA-issue bound: 64x64 output tiles, 4x4 register blocking per thread, operand
// tiles staged in shared memory with the per-row / per-column element offsets of the
// composite modes precomputed once per tile.
#include "common.cuh"

namespace jues {

namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

struct KArgs {
    long long M, N, K;
    double alpha, beta;
    const double *A; Mode mA, kA;
    const double *B; Mode kB, nB;
    double *C; Mode mC, nC;
    const double *Cin;
    long long mtiles;
    int a_mfast, b_nfast, c_mfast;
};

__global__ void __launch_bounds__(NT) gett_f64_kernel(KArgs g) {
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    __shared__ long long offA[BM], offB[BN], offCm[BM], offCn[BN];
    __shared__ long long koA[BK], koB[BK];

    const int tid = threadIdx.x;
    const long long tile = blockIdx.x;
    const long long m0 = (tile % g.mtiles) * BM;
    const long long n0 = (tile / g.mtiles) * BN;

    if (tid < BM) {
        long long m = m0 + tid;
        offA[tid] = m < g.M ? mode_off(g.mA, m) : -1;
        offCm[tid] = m < g.M ? mode_off(g.mC, m) : -1;
    } else if (tid < BM + BN) {
        long long n = n0 + tid - BM;
        offB[tid - BM] = n < g.N ? mode_off(g.nB, n) : -1;
        offCn[tid - BM] = n < g.N ? mode_off(g.nC, n) : -1;
    }

    // thread tile: 4 rows x 4 cols, strided by 16 to keep shared-memory reads conflict-free
    const int tr = g.c_mfast ? (tid & 15) : (tid >> 4);
    const int tc = g.c_mfast ? (tid >> 4) : (tid & 15);
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

    for (long long k0 = 0; k0 < g.K; k0 += BK) {
        __syncthreads();
        if (tid < BK) {
            long long k = k0 + tid;
            koA[tid] = k < g.K ? mode_off(g.kA, k) : -1;
        } else if (tid >= 32 && tid < 32 + BK) {
            long long k = k0 + tid - 32;
            koB[tid - 32] = k < g.K ? mode_off(g.kB, k) : -1;
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < (BM * BK) / NT; ++i) {
            int e = tid + i * NT;
            int m = g.a_mfast ? (e % BM) : (e / BK);
            int k = g.a_mfast ? (e / BM) : (e % BK);
            long long om = offA[m], ok = koA[k];
            As[k][m] = (om >= 0 && ok >= 0) ? __ldg(g.A + om + ok) : 0.0;
        }
#pragma unroll
        for (int i = 0; i < (BN * BK) / NT; ++i) {
            int e = tid + i * NT;
            int n = g.b_nfast ? (e % BN) : (e / BK);
            int k = g.b_nfast ? (e / BN) : (e % BK);
            long long on = offB[n], ok = koB[k];
            Bs[k][n] = (on >= 0 && ok >= 0) ? __ldg(g.B + on + ok) : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][tr + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tc + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        long long om = offCm[tr + 16 * i];
        if (om < 0) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            long long on = offCn[tc + 16 * j];
            if (on < 0) continue;
            double v = g.alpha * acc[i][j];
            if (g.beta != 0.0) v = fma(g.beta, g.Cin[om + on], v);
            g.C[om + on] = v;
        }
    }
}

// skinny GEMM (N <= 8): one warp per output row, lanes split K
__global__ void gett_f64_skinny(KArgs g) {
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= g.M) return;
    const long long m = warp;
    const long long om = mode_off(g.mA, m);
    double acc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] = 0.0;
    long long onb[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) onb[j] = j < g.N ? mode_off(g.nB, j) : 0;
    for (long long k = lane; k < g.K; k += 32) {
        const double a = __ldg(g.A + om + mode_off(g.kA, k));
        const long long ok = mode_off(g.kB, k);
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (j < g.N) acc[j] = fma(a, __ldg(g.B + ok + onb[j]), acc[j]);
    }
    const long long oc = mode_off(g.mC, m);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
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

}  // namespace

void gett_f64(Ctx *ctx, const GettArgs &a, const char *name) {
    if (a.M <= 0 || a.N <= 0) return;
    KArgs g;
    g.M = a.M; g.N = a.N; g.K = a.K;
    g.alpha = a.alpha; g.beta = a.beta;
    g.A = a.A; g.mA = a.mA; g.kA = a.kA;
    g.B = a.B; g.kB = a.kB; g.nB = a.nB;
    g.C = a.C; g.mC = a.mC; g.nC = a.nC;
    g.Cin = a.Cin ? a.Cin : a.C;
    g.mtiles = (a.M + BM - 1) / BM;
    long long ntiles = (a.N + BN - 1) / BN;
    g.a_mfast = (a.mA.s0 == 1 && a.mA.d0 > 1) ? 1 : 0;
    g.b_nfast = (a.nB.s0 == 1 && a.nB.d0 > 1) ? 1 : 0;
    g.c_mfast = (a.mC.s0 == 1 && a.mC.d0 > 1) ? 1 : 0;
    if (a.N <= 8) {
        long long blocks = (a.M * 32 + 255) / 256;
        JUES_REQUIRE(blocks < (1LL << 31), "GEMM too large for one launch");
        Ctx::Scope s(ctx, name);
        gett_f64_skinny<<<(unsigned)blocks, 256, 0, ctx->stream>>>(g);
        JUES_CHECK_CUDA(cudaGetLastError());
        return;
    }
    long long tiles = g.mtiles * ntiles;
    JUES_REQUIRE(tiles < (1LL << 31), "GEMM too large for one launch");
    Ctx::Scope s(ctx, name);
    gett_f64_kernel<<<(unsigned)tiles, NT, 0, ctx->stream>>>(g);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void gett(Ctx *ctx, int precision, const GettArgs &g, const char *name) {
    if (precision == JUES_PREC_SPLIT_BF16)
        gett_tc(ctx, g, name);
    else
        gett_f64(ctx, g, name);
}

}  // namespace jues
