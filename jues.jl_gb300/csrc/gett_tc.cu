// Split-precision GEMM over tensor modes on the sm_103a tensor cores (tcgen05 + TMEM + TMA).
//
// Each FP64 operand row r (a row of A or of B, running over K) is cut into chunks of KCH = 128
// K values (two pipeline stages); chunk c gets a power-of-two scale 2^e with max |x| < 2^e over
// the chunk, and every element is written as two integers carried exactly in FP16,
//     x = 2^(e - 9) (hi + 2^-10 lo),   hi = rint(x 2^(9 - e)),  |hi|, |lo| <= 512,
// so |x - 2^(e-9)(hi + 2^-10 lo)| <= 2^(e-20).  One CTA computes 128 x BN tiles of C = A.B^T
// with tcgen05.mma (kind::f16) products per K=16 step: hi.hi into a "main" TMEM accumulator and
// hi.lo + lo.hi into a "correction" accumulator (lo.lo, O(2^-20), is dropped).  Because the FP16
// values are integers, every product is exact and the main accumulator's partial sums over one
// chunk are exact FP32 integers while they stay below 2^24 (128 products of up to 2^18: random
// signs keep them near 2^21; only a chunk of equal-signed maximal products could pass 2^24,
// and then the tensor core's truncation costs at most one unit in 2^24 of that sum).  The
// correction term is 2^-10 smaller, so its rounding is below 1e-10 of the result.  Chunks
// alternate between two TMEM buffers; eight warps scale each finished chunk by
// 2^(e_r + e_c - 18) and add it into FP32 registers (round-to-nearest, unbiased) while the next
// chunk runs, then write the tile through the output tensor modes without the FP64 pipe
// (integer FP32 -> FP64 conversion, power-of-two alpha folded into the FP32 scale, in-place
// accumulation as L2 reductions).  The grid is persistent (one CTA per SM); a ragged last round
// has its tiles split over K, their parts summed by tail_reduce_kernel.  Operand tiles
// arrive by TMA (128-byte swizzle) into a STAGES-deep shared-memory ring guarded by mbarriers;
// one thread issues the TMA loads and one the MMAs.  Every mbarrier wait is bounded by
// %globaltimer; on expiry the CTA raises FLAG_TIMEOUT, skips its stores, frees its TMEM and
// returns.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "convert.cuh"

namespace jues {

namespace {

constexpr int TBM = 128;   // tile rows (TMEM lanes)
constexpr int TBK = 64;    // K elements per stage: 128 bytes of FP16 = one swizzle atom row
constexpr unsigned long long WAIT_LIMIT_NS = 2ull * 1000 * 1000 * 1000;    // 2 s: legitimate waits last microseconds

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// try_wait with a suspend-time hint: a waiting thread sleeps until the phase completes (or up to
// 20 us) instead of polling, which keeps the spinning warps off the shared-memory pipe the
// tensor cores read their operands through
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(20000u)
        : "memory");
    return ok != 0;
}
// bounded wait; false when the time limit expired, another thread of the CTA aborted, or
// another CTA already raised FLAG_TIMEOUT
__device__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                          const volatile unsigned *gflags) {
    unsigned long long t0 = 0;
    for (uint32_t it = 0;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 15u) == 15u) {
            if (*abort_flag || (*gflags & FLAG_TIMEOUT)) return false;
            unsigned long long t = gtimer();
            if (t0 == 0) t0 = t;
            else if (t - t0 > WAIT_LIMIT_NS) return false;
        }
    }
}
// bounded wait that ignores the abort flags: used only to let this CTA's own asynchronous
// copies and MMAs settle before it frees TMEM and exits
__device__ bool mbar_wait_quiet(uint64_t *bar, uint32_t parity) {
    unsigned long long t0 = 0;
    for (uint32_t it = 0;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 15u) == 15u) {
            unsigned long long t = gtimer();
            if (t0 == 0) t0 = t;
            else if (t - t0 > WAIT_LIMIT_NS) return false;
        }
    }
}
// a wait on a barrier phase that nothing completes: the bounded wait expires and the kernel
// raises FLAG_TIMEOUT, the failure path of every pipeline wait, exercised without a fault
__global__ void expired_wait_kernel(unsigned *flags) {
    __shared__ uint64_t bar;
    __shared__ int abort_flag;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0 && !mbar_wait(&bar, 0u, &abort_flag, flags)) atomicOr(flags, FLAG_TIMEOUT);
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y,
                                            int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// D[tmem] (+)= A[smem desc] . B[smem desc]^T, 16-bit inputs, FP32 accumulation
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}
// 32 lanes x 32 consecutive 32-bit TMEM columns -> 32 registers per thread
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// packed FP32 pairs (sm_100+): two round-to-nearest operations per instruction
__device__ __forceinline__ uint64_t pk2(uint32_t lo, uint32_t hi) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "r"(lo), "r"(hi));
    return r;
}
__device__ __forceinline__ uint64_t pk2f(float lo, float hi) { return pk2(__float_as_uint(lo), __float_as_uint(hi)); }
__device__ __forceinline__ uint64_t ffma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t fmul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ float lo_f(uint64_t x) { return __uint_as_float((uint32_t)x); }
__device__ __forceinline__ float hi_f(uint64_t x) { return __uint_as_float((uint32_t)(x >> 32)); }
__device__ __forceinline__ void red_add_f64(double *p, double v) {
    asm volatile("red.global.add.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}

// UMMA shared-memory descriptor of a K-major tile written by TMA with 128-byte swizzle:
// start address >> 4, LBO unused (1), SBO = 1024 bytes between 8-row groups, version 1,
// layout type 2 = SWIZZLE_128B.
__device__ __forceinline__ uint64_t sw128_desc(const void *smem) {
    const uint64_t a = smem_u32(smem);
    return ((a & 0x3FFFFull) >> 4) | (1ull << 16) | (64ull << 32) | (1ull << 46) | (2ull << 61);
}

struct TcArgs {
    long long M, N;        // logical GEMM extent (rows of A, rows of B)
    int kblocks;           // padded K / TBK
    long long mtiles;
    const int *expA, *expB;   // per-(chunk,row) power-of-two scales, [chunk][row]
    long long expA_ld, expB_ld;   // padded row counts (chunk strides)
    double alpha, beta;
    // Epilogue arithmetic without the FP64 pipe (about two operations per clock per SM on
    // GB300): alpha = (-1)^alpha_neg 2^alpha_k is folded into the FP32 row scale when
    // alpha_pow2; beta_mode 0: C = alpha AB; 1: C += alpha AB in place (Cin == C, beta == 1),
    // added by the L2's FP64 reduction unit; 2: C = Cin + alpha AB; 3: C = beta Cin + alpha AB.
    int alpha_pow2, alpha_k, alpha_neg, beta_mode;
    double *C;
    const double *Cin;
    Mode mC, nC;
    unsigned *flags;
    // split-K: CTA b computes tile b % tiles over stages [s kper, min(kblocks, (s+1) kper)),
    // s = b / tiles.  With ksplit > 1 the tile's FP32 sums go to partial[s][Npad][Mpad]
    // (rows contiguous) and splitk_reduce applies alpha and beta.
    long long tiles = 0;
    int ksplit = 1;
    int kper = 0;
    float *partial = nullptr;
    // Ragged last round (ksplit == 1): items [0, full_items) are whole tiles 0..full_items-1;
    // the tail_tiles tiles after them are split tail_ks ways over K (tail_kper stages each), so
    // the last round keeps every SM busy.  Their FP32 sums go to
    // tail_partial[split][tail tile][BN][TBM] and tail_reduce_kernel finishes them.
    long long full_items = 0;   // 0: no tail split
    int tail_tiles = 0, tail_ks = 1, tail_kper = 0;
    float *tail_partial = nullptr;
};

// one problem of a grouped launch (see gett_tc_kernel)
struct TcGroupProb {
    TcArgs a;
    int rowA, rowB;
    long long item0;
};

// Warp roles: warp 0 issues TMA, warp 1 owns TMEM and issues MMAs, warps 2-9 drain TMEM (two
// warps per 32-lane TMEM quarter, each owning half of the tile's columns).
// The MMA warp restarts both accumulators every KC stages (one scaling chunk of KCH = KC * 64
// K values), alternating between two TMEM buffers.
constexpr int TC_THREADS = 320;
constexpr int TC_DRAIN = 256;   // drain threads (warps 2-9)

__host__ __device__ constexpr uint32_t pow2_at_least(uint32_t x) {
    return x <= 32 ? 32u : (x <= 64 ? 64u : (x <= 128 ? 128u : (x <= 256 ? 256u : 512u)));
}
// instruction descriptor: FP32 accumulate, FP16 A and B (format 0), both K-major, M = 128, N = n
__host__ __device__ constexpr uint32_t tc_idesc(int n) {
    return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TBM >> 4) << 24);
}

// NP = operand planes: 2 (hi, lo) or 3 (hi, mid, lo)
template <int BN, int STAGES, int KC, int NP>
struct TcCfg {
    static constexpr int A_BYTES = TBM * TBK * 2;   // one plane
    static constexpr int B_BYTES = BN * TBK * 2;
    static constexpr int STAGE_BYTES = NP * A_BYTES + NP * B_BYTES;
    static constexpr int BAR_BYTES = 256;
    static constexpr int SMEM = STAGES * STAGE_BYTES + BAR_BYTES + BN * 8 + 2 * BN * 4 + 1024;
    static constexpr int BUF_COLS = NP * BN;   // one chunk buffer: NP accumulators of BN columns
    static constexpr uint32_t TMEM_COLS = pow2_at_least(2 * BUF_COLS);   // two chunk buffers
    static_assert(2 * BUF_COLS <= 512, "TMEM holds 512 columns");
    static_assert(NP * BN <= 256, "one MMA instruction spans at most N = 256");
};

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// output tile index -> (m0, n0).  Raster: groups of (up to) 16 row tiles, rows fastest within a
// group, so the CTAs resident at one time reuse a few row tiles' operand rows from L2 across
// about ten column tiles.
__device__ __forceinline__ void tc_tile_origin(const TcArgs &g, long long tile, int BN, int &m0, int &n0) {
    const long long G = min(g.mtiles, 16LL);
    const long long span = G * (g.tiles / g.mtiles);
    const long long grp = tile / span, in = tile - grp * span;
    const long long gm = min(G, g.mtiles - grp * G);
    m0 = (int)((grp * G + in % gm) * TBM);
    n0 = (int)((in / gm) * BN);
}

__host__ __device__ __forceinline__ long long tc_nitems(const TcArgs &g) {
    return g.full_items > 0 ? g.full_items + (long long)g.tail_tiles * g.tail_ks : g.tiles * g.ksplit;
}

// one work item of the persistent kernel: output tile (m0, n0) over stages [kb0, kb0 + nk);
// tail >= 0 marks a split part of a tail tile
struct TcItem {
    int m0, n0, kb0, nk;
    long long split;
    int tail;
};
__device__ __forceinline__ TcItem tc_item(const TcArgs &g, long long w, int BN) {
    TcItem I;
    long long tile;
    if (g.full_items > 0 && w >= g.full_items) {
        const long long u = w - g.full_items;
        I.tail = (int)(u % g.tail_tiles);
        I.split = u / g.tail_tiles;
        tile = g.full_items + I.tail;
        I.kb0 = (int)I.split * g.tail_kper;
        I.nk = min(g.kblocks - I.kb0, g.tail_kper);
    } else {
        I.tail = -1;
        tile = w % g.tiles;
        I.split = w / g.tiles;
        I.kb0 = (int)I.split * g.kper;
        I.nk = min(g.kblocks - I.kb0, g.kper);
    }
    tc_tile_origin(g, tile, BN, I.m0, I.n0);
    return I;
}

// barrier over the 256 drain threads (named barrier 1) that returns, uniformly to all of them,
// whether any thread passed pred = true
__device__ __forceinline__ bool drain_bar_any(bool pred) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, 1, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)pred), "n"(TC_DRAIN)
        : "memory");
    return r != 0;
}

// Column offsets of a thread's half tile: read from shared memory (any output mode), or
// computed for a single-stride column mode
struct ColsShared {
    const long long *co;
    __device__ __forceinline__ long long operator()(int j) const { return co[j]; }
};
struct ColsStrided {
    long long base, step;
    int nvalid;
    __device__ __forceinline__ long long operator()(int j) const { return j < nvalid ? base + j * step : -1; }
};

// One thread's row of an output tile: HB FP32 sums (column pairs packed in acc2) scaled and
// scattered through the output modes (co(j): column offsets, -1 past N).  Each form is its own
// loop, so no FP64 instruction is issued that the form does not need: POW2 (alpha folded into
// the FP32 scale) converts and stores only.  The conversion takes the short normal-or-zero
// form, and branches off for subnormal, infinite and NaN sums.
template <int HB, bool POW2, class Cols>
__device__ __forceinline__ void tc_epilogue(const TcArgs &g, const uint64_t *acc2, const Cols co, long long rowoff) {
    double *out = g.C + rowoff;
    auto value = [&](int j) {
        const float f = (j & 1) ? hi_f(acc2[j >> 1]) : lo_f(acc2[j >> 1]);
        const uint32_t a = __float_as_uint(f) & 0x7FFFFFFFu;
        double v;
        if (__builtin_expect((a - 1u < 0x7FFFFFu) | (a > 0x7F7FFFFFu), 0))
            v = f32_to_f64(f);   // subnormal, infinite or NaN
        else
            v = f32_to_f64_normal(f);
        if constexpr (POW2)
            return v;
        else
            return g.alpha * v;
    };
    if (g.beta_mode == 0) {
#pragma unroll
        for (int j = 0; j < HB; ++j)
            if (co(j) >= 0) out[co(j)] = value(j);
    } else if (g.beta_mode == 1) {
        // in-place sums as L2 reductions: one owner per element, so they are deterministic,
        // and round-to-nearest like the FP64 add they replace
#pragma unroll
        for (int j = 0; j < HB; ++j)
            if (co(j) >= 0) red_add_f64(out + co(j), value(j));
    } else {
        // Each output element is read and written by this thread alone, so a batch's inputs are
        // all loaded before any of its outputs is stored: the loads are in flight together
        // instead of one load latency per column (C and Cin may alias).
        const double *in = g.Cin + rowoff;
        constexpr int EB = HB < 16 ? HB : 16;
#pragma unroll
        for (int j0 = 0; j0 < HB; j0 += EB) {
            double cin[EB];
#pragma unroll
            for (int j = 0; j < EB; ++j) cin[j] = co(j0 + j) >= 0 ? __ldcs(in + co(j0 + j)) : 0.0;
            if (g.beta_mode == 2) {
#pragma unroll
                for (int j = 0; j < EB; ++j)
                    if (co(j0 + j) >= 0) out[co(j0 + j)] = cin[j] + value(j0 + j);
            } else {
#pragma unroll
                for (int j = 0; j < EB; ++j)
                    if (co(j0 + j) >= 0) out[co(j0 + j)] = fma(g.beta, cin[j], value(j0 + j));
            }
        }
    }
}


// GROUPED: the launch covers many independent problems (a batch), each with one K block
// (K <= 64); item w is output tile w - item0 of the problem whose [item0, next item0) holds it,
// its operand rows start at rowA / rowB of the concatenated planes that mapA / mapB describe, and
// g.tiles is the launch's total item count.
template <int BN, int STAGES, int KC, int NP, bool GROUPED>
__global__ void __launch_bounds__(TC_THREADS, 1)
    gett_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                   const __grid_constant__ TcArgs g, const TcGroupProb *__restrict__ gp, int ngp) {
    using Cfg = TcCfg<BN, STAGES, KC, NP>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *stages = smem;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * Cfg::STAGE_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *cfull = empty + STAGES;    // [2] chunk accumulated in TMEM buffer
    uint64_t *cempty = cfull + 2;        // [2] chunk drained, buffer reusable
    uint64_t *fin = cempty + 2;          // the MMA thread's last commit
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(fin + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    long long *coloff = reinterpret_cast<long long *>(smem + STAGES * Cfg::STAGE_BYTES + Cfg::BAR_BYTES);
    float *colsc = reinterpret_cast<float *>(coloff + BN);   // [2][BN] per-chunk column scales

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // persistent: CTA b processes work items b, b + gridDim.x, ...; an item is one output tile
    // over one K split.  Stage and chunk counters run on across items, so the pipeline and the
    // TMEM buffers never drain between tiles.
    const long long nitems = GROUPED ? g.tiles : tc_nitems(g);
    // the problem of item w, its tile and its operand row offsets
    auto locate = [&](long long w, const TcArgs *&G, int &ra, int &rb) -> TcItem {
        if constexpr (GROUPED) {
            int lo = 0, hi = ngp - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (gp[mid].item0 <= w) lo = mid; else hi = mid - 1;
            }
            G = &gp[lo].a;
            ra = gp[lo].rowA;
            rb = gp[lo].rowB;
            return tc_item(*G, w - gp[lo].item0, BN);
        } else {
            G = &g;
            ra = rb = 0;
            return tc_item(g, w, BN);
        }
    };

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&cfull[b], 1);
            mbar_init(&cempty[b], TC_DRAIN);
        }
        mbar_init(fin, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        tmem_alloc(tmem_slot, Cfg::TMEM_COLS);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // TMA producer
            long long it = 0;   // stages issued by this CTA
            bool stop = false;
            for (long long w = blockIdx.x; w < nitems && !stop; w += gridDim.x) {
                const TcArgs *G;
                int ra, rb;
                const TcItem I = locate(w, G, ra, rb);
                for (int kb = 0; kb < I.nk; ++kb, ++it) {
                    const int s = (int)(it % STAGES);
                    const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                    if (!mbar_wait(&empty[s], ph ^ 1u, abort_flag, g.flags)) {
                        *abort_flag = 1;
                        stop = true;
                        break;
                    }
                    uint8_t *st = stages + s * Cfg::STAGE_BYTES;
                    const int kx = (I.kb0 + kb) * TBK;
                    mbar_expect_tx(&full[s], Cfg::STAGE_BYTES);
#pragma unroll
                    for (int p = 0; p < NP; ++p)
                        tma_load_3d(st + p * Cfg::A_BYTES, &mapA, &full[s], kx, I.m0 + ra, p);
#pragma unroll
                    for (int p = 0; p < NP; ++p)
                        tma_load_3d(st + NP * Cfg::A_BYTES + p * Cfg::B_BYTES, &mapB, &full[s], kx, I.n0 + rb, p);
                }
            }
            // the last load into each slot has landed (immediate unless an abort cut the MMA
            // thread short), so no copy is in flight when the CTA exits
            for (int s = 0; s < STAGES; ++s)
                if (it > s) {
                    const long long last = s + ((it - 1 - s) / STAGES) * STAGES;
                    mbar_wait_quiet(&full[s], (uint32_t)(last / STAGES) & 1u);
                }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer: chunk gc (counted across items) accumulates into TMEM buffer gc & 1
            long long it = 0, gc = 0;
            bool stop = false;
            for (long long w = blockIdx.x; w < nitems && !stop; w += gridDim.x) {
                const TcArgs *G;
                int ra, rb;
                const TcItem I = locate(w, G, ra, rb);
                for (int kb = 0; kb < I.nk; ++kb, ++it) {
                    const int buf = (int)(gc & 1);
                    const bool first = (kb % KC) == 0;
                    if (first && gc >= 2) {
                        if (!mbar_wait(&cempty[buf], (uint32_t)((gc >> 1) - 1) & 1u, abort_flag, g.flags)) {
                            *abort_flag = 1;
                            stop = true;
                            break;
                        }
                        tc_fence_after();
                    }
                    const int s = (int)(it % STAGES);
                    const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                    if (!mbar_wait(&full[s], ph, abort_flag, g.flags)) {
                        *abort_flag = 1;
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    uint8_t *st = stages + s * Cfg::STAGE_BYTES;
                    const uint64_t b0 = sw128_desc(st + NP * Cfg::A_BYTES);
                    const uint32_t dbuf = tmem + (uint32_t)(buf * Cfg::BUF_COLS);
                    // The B planes' rows are stacked in shared memory (B_BYTES = BN 128-byte rows,
                    // whole 8-row swizzle groups) and the NP accumulators of a buffer are adjacent
                    // TMEM column ranges, so plane p of A against B planes 0..NP-1-p is one
                    // instruction with N = (NP - p) BN writing accumulators p..NP-1: accumulator
                    // j collects every product A_p B_q with p + q = j (j < NP), and the products
                    // with p + q >= NP (lo.lo, 2^-20 or 2^-30 smaller) are left out.
#pragma unroll
                    for (int kk = 0; kk < TBK / 16; ++kk) {
                        const uint64_t off = (uint64_t)((kk * 16 * 2) >> 4);   // 32 bytes per K=16 step
                        const uint32_t acc = (first && kk == 0) ? 0u : 1u;
#pragma unroll
                        for (int p = 0; p < NP; ++p)
                            umma_bf16(dbuf + (uint32_t)(p * BN), sw128_desc(st + p * Cfg::A_BYTES) + off, b0 + off,
                                      tc_idesc((NP - p) * BN), p == 0 ? acc : 1u);
                    }
                    umma_commit(&empty[s]);   // stage s free once these complete
                    if ((kb % KC) == KC - 1 || kb == I.nk - 1) {
                        umma_commit(&cfull[buf]);   // chunk done
                        ++gc;
                    }
                }
            }
            // every MMA this thread issued has completed before TMEM is freed
            umma_commit(fin);
            mbar_wait_quiet(fin, 0u);
        }
    } else {
        // drain warps 2-9: TMEM lane quarter (warp % 4), one tile row per thread, half the columns.
        // They leave their loops only together: every exit test follows a barrier that ORs the
        // threads' failure flags, so no drain thread can be left waiting at a barrier.
        constexpr int HB = BN / 2;
        const int quarter = warp & 3;
        const int half = (warp - 2) >> 2;
        const int dt = threadIdx.x - 64;   // 0..255 among the drain threads
        long long gc = 0;
        bool ok = true;
        for (long long w = blockIdx.x; w < nitems; w += gridDim.x) {
            const TcArgs *G;
            int ra, rb;
            const TcItem I = locate(w, G, ra, rb);
            const int nchunks = (I.nk + KC - 1) / KC;
            const int chunk0 = I.kb0 / KC;   // kper is a multiple of KC
            // every drain thread has finished the previous item's epilogue (which reads coloff)
            if (drain_bar_any(*abort_flag != 0)) {
                ok = false;
                break;
            }
            if (dt < BN) {
                const long long n = (long long)I.n0 + dt;
                coloff[dt] = n < G->N ? mode_off(G->nC, n) : -1;
            }
            uint64_t acc2[HB / 2];   // FP32 pairs (columns 2j, 2j+1)
#pragma unroll
            for (int j = 0; j < HB / 2; ++j) acc2[j] = 0ull;
            const long long mrow = (long long)I.m0 + quarter * 32 + lane;
            // the scales of chunk c + 1 are loaded while chunk c drains
            const int *pa = G->expA + (long long)chunk0 * G->expA_ld + mrow;
            const int *pb = G->expB + (long long)chunk0 * G->expB_ld + I.n0 + (dt < BN ? dt : 0);
            int ea_cur = __ldg(pa), eb_cur = __ldg(pb);
            bool bad = false;
            for (int c = 0; c < nchunks; ++c, ++gc) {
                const int buf = (int)(gc & 1);
                // column scales of this chunk: 2^e_col, staged once for all drain warps
                if (dt < BN)
                    colsc[buf * BN + dt] =
                        (eb_cur == INT_MIN || eb_cur < -126) ? 0.f : __int_as_float((eb_cur + 127) << 23);
                int ea_next = 0, eb_next = 0;
                if (c + 1 < nchunks) {
                    ea_next = __ldg(pa + (long long)(c + 1) * G->expA_ld);
                    eb_next = __ldg(pb + (long long)(c + 1) * G->expB_ld);
                }
                if (drain_bar_any(bad || *abort_flag != 0)) {
                    bad = true;
                    break;
                }
                // warp-uniform outcome: the TMEM loads below need the whole warp
                const bool got = mbar_wait(&cfull[buf], (uint32_t)(gc >> 1) & 1u, abort_flag, g.flags);
                if (!__all_sync(0xffffffffu, got)) {
                    *abort_flag = 1;
                    bad = true;   // the next barrier takes every drain thread out
                    continue;
                }
                __syncwarp();
                tc_fence_after();
                const int ea = ea_cur;
                ea_cur = ea_next;
                eb_cur = eb_next;
                // row factor 2^(e_row - 18) (times alpha when that is a power of two); the column
                // factor comes from shared memory
                const int er = ea - 18 + G->alpha_k;
                const float rs = (ea == INT_MIN || er < -126)
                                     ? 0.f
                                     : __int_as_float((er + 127) << 23 | (G->alpha_neg ? 0x80000000 : 0));
                const float2 *cs = reinterpret_cast<const float2 *>(colsc + buf * BN + half * HB);
                const uint64_t rs2 = pk2f(rs, rs), k2 = pk2f(0.0009765625f, 0.0009765625f);
                // 32 columns per round: the NP accumulator loads in flight, one wait; then per
                // column pair part = main + 2^-10 (corr + 2^-10 corr2), acc += part (2^e_row 2^e_col),
                // all round-to-nearest
#pragma unroll
                for (int c0 = 0; c0 < HB; c0 += 32) {
                    uint32_t r0[32], r1[32], r2[NP > 2 ? 32 : 1];
                    const uint32_t base = tmem + ((uint32_t)(quarter * 32) << 16) +
                                          (uint32_t)(buf * Cfg::BUF_COLS + half * HB + c0);
                    tmem_ld32(base, r0);
                    tmem_ld32(base + (uint32_t)BN, r1);
                    if constexpr (NP > 2) tmem_ld32(base + (uint32_t)(2 * BN), *reinterpret_cast<uint32_t(*)[32]>(r2));
                    tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 32; j += 2) {
                        const float2 c2 = cs[(c0 + j) >> 1];
                        uint64_t corr = pk2(r1[j], r1[j + 1]);
                        if constexpr (NP > 2) corr = ffma2(pk2(r2[j], r2[j + 1]), k2, corr);
                        const uint64_t part = ffma2(corr, k2, pk2(r0[j], r0[j + 1]));
                        const uint64_t sc = fmul2(rs2, pk2f(c2.x, c2.y));
                        acc2[(c0 + j) >> 1] = ffma2(part, sc, acc2[(c0 + j) >> 1]);
                    }
                }
                tc_fence_before();
                mbar_arrive(&cempty[buf]);
            }
            if (drain_bar_any(bad)) {   // every drain thread takes part, failed or not
                ok = false;
                break;
            }
            if (I.tail >= 0) {
                // a split part of a tail tile: raw sums (alpha folded in when a power of two),
                // [split][tail tile][column][row], a warp writing 32 consecutive floats
                float *dst = G->tail_partial + (((long long)I.split * G->tail_tiles + I.tail) * BN + half * HB) * TBM +
                             quarter * 32 + lane;
#pragma unroll
                for (int j = 0; j < HB / 2; ++j) {
                    dst[(long long)(2 * j) * TBM] = lo_f(acc2[j]);
                    dst[(long long)(2 * j + 1) * TBM] = hi_f(acc2[j]);
                }
            } else if (G->partial) {
                // raw partial sums, padded rows and columns included; a warp writes 32
                // consecutive floats per column
                const long long Mpad = G->mtiles * TBM, Npad = (G->tiles / G->mtiles) * BN;
                float *dst = G->partial + ((long long)I.split * Npad + I.n0 + half * HB) * Mpad + mrow;
#pragma unroll
                for (int j = 0; j < HB / 2; ++j) {
                    dst[(long long)(2 * j) * Mpad] = lo_f(acc2[j]);
                    dst[(long long)(2 * j + 1) * Mpad] = hi_f(acc2[j]);
                }
            } else if (mrow < G->M) {
                const long long rowoff = mode_off(G->mC, mrow);
                const long long n1 = (long long)I.n0 + half * HB;
                if (G->nC.d0 == MODE_BIG) {
                    const ColsStrided cols{n1 * G->nC.s0, G->nC.s0, (int)max(-1LL, min((long long)HB, G->N - n1))};
                    if (G->alpha_pow2)
                        tc_epilogue<HB, true>(*G, acc2, cols, rowoff);
                    else
                        tc_epilogue<HB, false>(*G, acc2, cols, rowoff);
                } else {
                    const ColsShared cols{coloff + half * HB};
                    if (G->alpha_pow2)
                        tc_epilogue<HB, true>(*G, acc2, cols, rowoff);
                    else
                        tc_epilogue<HB, false>(*G, acc2, cols, rowoff);
                }
            }
        }
        if (!ok && lane == 0) atomicOr(g.flags, FLAG_TIMEOUT);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, Cfg::TMEM_COLS);
    }
}

// The split parts of the tail tiles, summed in split order in FP64 (deterministic), then
// alpha (unless folded into the parts), beta and the output modes.  Grid (TBM BN / 256, tail
// tiles): one element per thread, consecutive threads on consecutive rows (coalesced), the
// parts of an element loaded before they are summed.
__global__ void __launch_bounds__(256) tail_reduce_kernel(const TcArgs g, int BN) {
    const int q = blockIdx.y;
    const int e = blockIdx.x * 256 + threadIdx.x;
    const int r = e % TBM, c = e / TBM;
    int m0, n0;
    tc_tile_origin(g, g.full_items + q, BN, m0, n0);
    const long long m = (long long)m0 + r, n = (long long)n0 + c;
    if (c >= BN || m >= g.M || n >= g.N) return;
    const float *p = g.tail_partial + ((long long)q * BN + c) * TBM + r;
    const long long sstride = (long long)g.tail_tiles * BN * TBM;
    float part[16];
#pragma unroll
    for (int s = 0; s < 16; ++s) part[s] = s < g.tail_ks ? p[s * sstride] : 0.f;
    double acc = 0.0;
#pragma unroll
    for (int s = 0; s < 16; ++s)
        if (s < g.tail_ks) acc += to_f64(part[s]);
    const long long off = mode_off(g.mC, m) + mode_off(g.nC, n);
    double v = (g.alpha_pow2 || g.alpha == 1.0) ? acc : g.alpha * acc;
    if (g.beta != 0.0) v = fma(g.beta, g.Cin[off], v);
    g.C[off] = v;
}

constexpr int PR = 16, PK = 128, KCH = 128;   // pack tile = one scaling chunk = two pipeline stages

// FP64 operand -> integer-valued FP16 planes [NP][Rpad][Kpad], K-major, and the per-(chunk,row)
// scales, in one pass.  A block covers 16 rows x one 128-wide K chunk (the last chunk may be 64
// wide: Kpad is a multiple of 64), so the chunk maximum is a block-local reduction.  Each
// thread loads 8 elements (4 column pairs of one row when the source's rows are unit-stride,
// one column pair of 4 rows when its K is) and keeps them in registers: the row maxima go
// through shared-memory atomics, the planes are staged in shared memory as FP16 pairs and
// written out as 8-byte pieces of 256-byte rows.  The split works on the IEEE-754 bit pattern
// with integer arithmetic only (GB300 runs FP64 arithmetic at a small fraction of its integer
// rate): for x = +-m 2^(E-1075) (m the 53-bit significand) and chunk scale e,
//     q = rint(x 2^(19-e)) = round(m >> (1056 + e - E)),  hi = (q + 512) >> 10,  lo = q - 1024 hi,
// so x ~ 2^(e-19) q = 2^(e-9) (hi + 2^-10 lo) with |hi| <= 512, |lo| <= 512.  The three-plane
// form keeps 29 bits: q = rint(x 2^(29-e)) = 2^20 hi + 2^10 mid + lo, x ~ 2^(e-9) (hi + 2^-10 mid
// + 2^-20 lo), |x - that| <= 2^(e-30).  Every element of the padded tile and every scale is
// written, so nothing has to be cleared beforehand.
__device__ __forceinline__ int exp_field(double x) {
    // biased exponent: 0 for zero and subnormals, which are flushed
    return (int)(((unsigned)__double2hiint(x) >> 20) & 0x7FFu);
}
// q = rint(x 2^(bits - e)), ties away from zero, for |x| < 2^e: bits = 19 (two planes) or 29
// (three planes).  With x = +-m 2^(E-1075), q = floor((m + 2^(r-1)) / 2^r), r = 1075 - bits + e - E
// >= 54 - bits, which equals floor((floor(m / 2^(r-1)) + 1) / 2) and needs only the top 32
// bits of m (m >> 21), so the whole split runs in 32-bit integer arithmetic.
__device__ __forceinline__ int fixed_q(double x, int e, int bits) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const int E = (int)((hi >> 20) & 0x7FFu);
    if (E == 0 || e == INT_MIN) return 0;
    const int sh = 1075 - bits + e - E - 22;   // r - 22 >= 32 - bits > 0
    if (sh >= 32) return 0;
    const unsigned mh = (((hi & 0xFFFFFu) | 0x100000u) << 11) | (lo >> 21);   // m >> 21
    const int q = (int)(((mh >> sh) + 1u) >> 1);
    return (hi >> 31) ? -q : q;
}
// the NP plane digits of q, each an integer in [-512, 512] (exact in FP16)
template <int NP>
__device__ __forceinline__ void split_digits(int q, int (&d)[NP]) {
    if constexpr (NP == 2) {
        const int h = (q + 512) >> 10;   // arithmetic shift: floor
        d[0] = h;
        d[1] = q - h * 1024;
    } else {
        const int h = (q + (1 << 19)) >> 20;
        const int rem = q - h * 1048576;
        const int m = (rem + 512) >> 10;
        d[0] = h;
        d[1] = m;
        d[2] = rem - m * 1024;
    }
}
__device__ __forceinline__ uint32_t half_pair(int a, int b) {
    const __half2 h = __halves2half2(__int2half_rn(a), __int2half_rn(b));
    return *reinterpret_cast<const uint32_t *>(&h);
}

// staged row pitch in 32-bit words (two FP16 each): 66 keeps the pair stores of both thread
// layouts free of bank conflicts and the 8-byte row pieces aligned
constexpr int PACK_PITCH = PK / 2 + 2;

// One pack block: rows [r0, r0 + 16) x K chunk [k0, k0 + 128) of one operand.  KFAST: the
// source's K index is unit-stride (else its row index is).  The planes go to
// dst[plane pstride + row Kld + k], the scales to rexp[(k0 / 128) rexp_ld + row].
template <int NP, bool KFAST>
__device__ __forceinline__ void pack_block(const double *__restrict__ src, const Mode &rmode, const Mode &kmode,
                                           long long R, long long K, long long Kpad, long long r0, long long k0,
                                           int *__restrict__ rexp, long long rexp_ld, __half *__restrict__ dst,
                                           long long pstride, long long Kld, double scale = 1.0) {
    __shared__ __align__(16) uint32_t outp[NP][PR][PACK_PITCH];
    __shared__ long long roff[PR], koff[PK];
    __shared__ int rowE[PR];
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid < PR) {
        const long long r = r0 + tid;
        roff[tid] = r < R ? mode_off(rmode, r) : -1;
        rowE[tid] = 0;
    } else if (tid >= 64 && tid < 64 + PK) {
        const long long k = k0 + tid - 64;
        koff[tid - 64] = k < K ? mode_off(kmode, k) : -1;
    }
    __syncthreads();
    // element (i, h): row row_of(i), column 2 pair_of(i) + h
    auto row_of = [&](int i) { return KFAST ? (tid >> 6) + 4 * i : (tid & 15); };
    auto pair_of = [&](int i) { return KFAST ? (tid & 63) : (tid >> 4) + 16 * i; };
    double x[4][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const long long a = roff[row_of(i)], b = koff[2 * pair_of(i) + h];
            x[i][h] = (a >= 0 && b >= 0) ? __ldg(src + a + b) : 0.0;
        }
    if (scale != 1.0) {   // a power of two: exact
#pragma unroll
        for (int i = 0; i < 4; ++i) { x[i][0] *= scale; x[i][1] *= scale; }
    }
    // row maxima of the exponent field
    if constexpr (KFAST) {
        // a warp's lanes share each of its four rows
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int m = __reduce_max_sync(0xffffffffu, max(exp_field(x[i][0]), exp_field(x[i][1])));
            if (lane == 0) atomicMax(&rowE[row_of(i)], m);
        }
    } else {
        // all eight elements share the thread's row; lanes l and l + 16 share a row
        int m = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) m = max(m, max(exp_field(x[i][0]), exp_field(x[i][1])));
        m = max(m, __shfl_xor_sync(0xffffffffu, m, 16));
        if (lane < 16) atomicMax(&rowE[lane], m);
    }
    __syncthreads();
    if (tid < PR) {
        const int E = rowE[tid];
        rexp[(k0 / KCH) * rexp_ld + r0 + tid] = E == 0 ? INT_MIN : E - 1022;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = row_of(i);
        const int E = rowE[r];
        const int e = E == 0 ? INT_MIN : E - 1022;
        int d0[NP], d1[NP];
        split_digits<NP>(fixed_q(x[i][0], e, 10 * NP - 1), d0);
        split_digits<NP>(fixed_q(x[i][1], e, 10 * NP - 1), d1);
#pragma unroll
        for (int p = 0; p < NP; ++p) outp[p][r][pair_of(i)] = half_pair(d0[p], d1[p]);
    }
    __syncthreads();
    // NP planes x PR rows x 32 pieces of 4 halves
#pragma unroll
    for (int j = 0; j < (NP * PR * 32) / 256; ++j) {
        const int idx = tid + 256 * j;
        const int seg = idx & 31, row = (idx >> 5) & (PR - 1), plane = idx >> 9;
        const long long k = k0 + 4 * seg;
        if (k >= Kpad) continue;   // the 64-wide tail of the last chunk (Kpad is a multiple of 64)
        *reinterpret_cast<uint2 *>(dst + (size_t)plane * pstride + (size_t)(r0 + row) * Kld + k) =
            *reinterpret_cast<const uint2 *>(&outp[plane][row][2 * seg]);
    }
}

template <int NP, bool KFAST>
__global__ void __launch_bounds__(256, 6) pack_split_kernel(const double *__restrict__ src, Mode rmode, Mode kmode,
                                                         long long R, long long K, long long Rpad,
                                                         long long Kpad, int *__restrict__ rexp,
                                                         __half *__restrict__ dst, long long Kld,
                                                         long long pstride, double scale, long long rexp_ld) {
    // consecutive blocks follow the source's unit-stride index, so the blocks resident at one
    // time read long contiguous runs of it
    // block counts < 2^31 (checked at launch): 32-bit index arithmetic
    const unsigned kblocks = (unsigned)((Kpad + PK - 1) / PK), rblocks = (unsigned)(Rpad / PR);
    const long long r0 = (long long)(KFAST ? blockIdx.x / kblocks : blockIdx.x % rblocks) * PR;
    const long long k0 = (long long)(KFAST ? blockIdx.x % kblocks : blockIdx.x / rblocks) * PK;
    pack_block<NP, KFAST>(src, rmode, kmode, R, K, Kpad, r0, k0, rexp, rexp_ld, dst, pstride, Kld, scale);
}

// Grouped form: many operands (one per problem of a batch) with one 64-wide K block each
// (K <= 64), their rows concatenated into one set of planes [NP][rows][64] so that one tensor
// map covers all of them.  Problem p's rows start at row0, its blocks at block0.
struct PackProb {
    const double *src;
    Mode r, k;
    long long R, K, Rpad, row0, block0;
};
template <int NP>
__global__ void __launch_bounds__(256, 6) pack_grouped_kernel(const PackProb *__restrict__ probs, int nprob,
                                                              long long rows_total, int *__restrict__ rexp,
                                                              __half *__restrict__ dst) {
    const long long b = blockIdx.x;
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (probs[mid].block0 <= b) lo = mid; else hi = mid - 1;
    }
    const PackProb &P = probs[lo];
    const long long r0 = (b - P.block0) * PR;
    // the unit-stride choice is uniform over a block
    if (P.k.s0 == 1 && P.k.d0 > 1)
        pack_block<NP, true>(P.src, P.r, P.k, P.R, P.K, 64, r0, 0, rexp + P.row0, rows_total, dst + P.row0 * 64,
                             rows_total * 64, 64);
    else
        pack_block<NP, false>(P.src, P.r, P.k, P.R, P.K, 64, r0, 0, rexp + P.row0, rows_total, dst + P.row0 * 64,
                              rows_total * 64, 64);
}

// Pack rows [0, Rpad) x K [0, Kpad) of one operand into planes of row pitch Kld (plane stride
// pstride) and the [chunk][row] scales ex (chunk stride Rpad), each value times scale (a power of
// two); the plain packs have Kld = Kpad and pstride = Rpad Kpad.
template <int NP>
void launch_pack(Ctx *ctx, const double *src, const Mode &rm, const Mode &km, long long R, long long K,
                 long long Rpad, long long Kpad, int *ex, __half *dst, long long Kld = -1, long long pstride = -1,
                 double scale = 1.0, long long rexp_ld = -1) {
    if (Kld < 0) Kld = Kpad;
    if (pstride < 0) pstride = Rpad * Kpad;
    if (rexp_ld < 0) rexp_ld = Rpad;
    const long long blocks = (Rpad / PR) * ((Kpad + PK - 1) / PK);
    JUES_REQUIRE(blocks < (1LL << 31), "operand too large to pack in one launch");
    if (km.s0 == 1 && km.d0 > 1)
        pack_split_kernel<NP, true><<<(unsigned)blocks, 256, 0, ctx->stream>>>(src, rm, km, R, K, Rpad, Kpad, ex, dst,
                                                                               Kld, pstride, scale, rexp_ld);
    else
        pack_split_kernel<NP, false><<<(unsigned)blocks, 256, 0, ctx->stream>>>(src, rm, km, R, K, Rpad, Kpad, ex,
                                                                                dst, Kld, pstride, scale, rexp_ld);
    JUES_CHECK_CUDA(cudaGetLastError());
}


PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        JUES_CHECK_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !p)
            throw Error(JUES_ECUDA, "cuTensorMapEncodeTiled is not available from the driver");
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// planes [np][rows_pad][pitch] of FP16 digits, K columns [0, kpad) read (pitch >= kpad)
CUtensorMap make_map(const __half *base, long long rows_pad, long long kpad, int box_rows, int np,
                     long long pitch = -1) {
    if (pitch < 0) pitch = kpad;
    CUtensorMap m;
    std::memset(&m, 0, sizeof(m));
    cuuint64_t dims[3] = {(cuuint64_t)kpad, (cuuint64_t)rows_pad, (cuuint64_t)np};
    cuuint64_t strides[2] = {(cuuint64_t)pitch * 2, (cuuint64_t)rows_pad * pitch * 2};
    cuuint32_t box[3] = {(cuuint32_t)TBK, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = get_encode()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, const_cast<__half *>(base), dims,
                              strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(JUES_ECUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
    return m;
}

long long roundup(long long x, long long m) { return (x + m - 1) / m * m; }

bool same_mode(const Mode &a, const Mode &b) {
    return a.d0 == b.d0 && a.d1 == b.d1 && a.s0 == b.s0 && a.s1 == b.s1 && a.s2 == b.s2;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// packed-operand cache: scratch planes for transient operands, persistent planes for
// operands declared constant (integrals), dropped explicitly.
// ---------------------------------------------------------------------------------------
struct PackEntry {
    const double *src;
    Mode r, k;
    long long R, K, Rpad, Kpad;
    int np;
    DBuf<__half> buf;
    DBuf<int> exps;
};
struct PackCache {
    bool busy = false;   // inside a cache operation: frees of the cache's own buffers are not lookups
    std::vector<std::unique_ptr<PackEntry>> cached;
    DBuf<__half> scratch[2];
    DBuf<int> scratch_exp[2];
    // buffers of dropped entries, reused by later entries (no cudaFree/cudaMalloc per sweep)
    std::vector<DBuf<__half>> free_planes;
    std::vector<DBuf<int>> free_exps;
};

template <class T>
static DBuf<T> take_buffer(Ctx *ctx, std::vector<DBuf<T>> &pool, size_t need) {
    int best = -1;
    for (int i = 0; i < (int)pool.size(); ++i)
        if (pool[i].n >= need && (best < 0 || pool[i].n < pool[best].n)) best = i;
    if (best >= 0 && pool[best].n <= 2 * need) {
        DBuf<T> b = std::move(pool[best]);
        pool.erase(pool.begin() + best);
        return b;
    }
    return DBuf<T>(ctx, need);
}
struct Packed {
    const __half *planes;
    const int *exps;
};

void pack_cache_destroy(PackCache *p) {
    if (p) p->busy = true;
    delete p;
}
void pack_cache_clear(Ctx *ctx) {
    if (ctx->pack) {
        ctx->pack->busy = true;
        ctx->pack->cached.clear();
        ctx->pack->free_planes.clear();
        ctx->pack->free_exps.clear();
        ctx->pack->busy = false;
    }
}
// Entries are keyed by their source address.  Device memory is reused quickly (the context's
// pool hands freed blocks out again), so every free of device memory forgets the entries whose
// source lay in the freed range: a later array at the same address can never hit a stale pack.
void pack_cache_forget(Ctx *ctx, const void *p, size_t bytes) {
    if (!ctx->pack || ctx->pack->busy || !p) return;
    PackCache &pc = *ctx->pack;
    const char *b = static_cast<const char *>(p), *e = b + bytes;
    auto inside = [&](const std::unique_ptr<PackEntry> &x) {
        const char *q = reinterpret_cast<const char *>(x->src);
        return q >= b && q < e;
    };
    bool any = false;
    for (auto &x : pc.cached) any = any || inside(x);
    if (!any) return;
    pc.busy = true;
    for (auto &x : pc.cached)
        if (inside(x)) {
            pc.free_planes.push_back(std::move(x->buf));
            pc.free_exps.push_back(std::move(x->exps));
        }
    pc.cached.erase(std::remove_if(pc.cached.begin(), pc.cached.end(), inside), pc.cached.end());
    pc.busy = false;
}
void pack_cache_drop(Ctx *ctx, const void *ptr) {
    if (!ctx->pack) return;
    PackCache &pc = *ctx->pack;
    auto &v = pc.cached;
    for (auto &e : v)
        if (e->src == ptr) {
            pc.free_planes.push_back(std::move(e->buf));
            pc.free_exps.push_back(std::move(e->exps));
        }
    v.erase(std::remove_if(v.begin(), v.end(), [&](const std::unique_ptr<PackEntry> &e) { return e->src == ptr; }),
            v.end());
}

static Packed pack_operand(Ctx *ctx, int slot, const double *src, const Mode &rm, const Mode &km, long long R,
                           long long K, long long Rpad, long long Kpad, bool cache, int np) {
    if (!ctx->pack) ctx->pack = new PackCache();
    PackCache &pc = *ctx->pack;
    if (cache) {
        for (auto &e : pc.cached)
            if (e->src == src && e->R == R && e->K == K && e->Rpad == Rpad && e->Kpad == Kpad && e->np == np &&
                same_mode(e->r, rm) && same_mode(e->k, km))
                return Packed{e->buf.p, e->exps.p};
    }
    const size_t need = (size_t)np * Rpad * Kpad;
    const long long nchunk = (Kpad + KCH - 1) / KCH;
    __half *dst;
    int *ex;
    std::unique_ptr<PackEntry> ent;
    struct Busy {
        PackCache &c;
        explicit Busy(PackCache &x) : c(x) { c.busy = true; }
        ~Busy() { c.busy = false; }
    } busy(pc);
    if (cache) {
        ent.reset(new PackEntry{src, rm, km, R, K, Rpad, Kpad, np, take_buffer(ctx, pc.free_planes, need),
                                take_buffer(ctx, pc.free_exps, (size_t)nchunk * Rpad)});
        dst = ent->buf.p;
        ex = ent->exps.p;
    } else {
        if (pc.scratch[slot].n < need) {
            pc.scratch[slot].reset();
            pc.scratch[slot] = DBuf<__half>(ctx, need);
        }
        if (pc.scratch_exp[slot].n < (size_t)(nchunk * Rpad)) {
            pc.scratch_exp[slot].reset();
            pc.scratch_exp[slot] = DBuf<int>(ctx, (size_t)(nchunk * Rpad));
        }
        dst = pc.scratch[slot].p;
        ex = pc.scratch_exp[slot].p;
    }
    {
        Ctx::Scope s(ctx, "pack_split");
        if (np == 3)
            launch_pack<3>(ctx, src, rm, km, R, K, Rpad, Kpad, ex, dst);
        else
            launch_pack<2>(ctx, src, rm, km, R, K, Rpad, Kpad, ex, dst);
    }
    if (cache) pc.cached.push_back(std::move(ent));
    return Packed{dst, ex};
}

constexpr int TC_KC = KCH / TBK;   // stages per accumulation chunk (one scaling chunk)

static int sm_count(int device) {
    static int cached[64] = {};
    if (device < 0 || device >= 64) return 148;
    if (!cached[device]) {
        int n = 0;
        JUES_CHECK_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device));
        cached[device] = n > 0 ? n : 148;
    }
    return cached[device];
}

template <int BN, int STAGES, int NP>
static void launch_tc(Ctx *ctx, const CUtensorMap &ma, const CUtensorMap &mb, const TcArgs &t, long long tiles,
                      const char *name, bool allow_tail = true) {
    using Cfg = TcCfg<BN, STAGES, TC_KC, NP>;
    // the shared-memory limit is a per-device attribute of the kernel: set once on every device
    // this instantiation launches on (the calling entry point made ctx->device current)
    static std::atomic<unsigned long long> attr_set{0};
    const unsigned long long bit = ctx->device >= 0 && ctx->device < 64 ? 1ull << ctx->device : 0ull;
    if (!bit || !(attr_set.load() & bit)) {
        JUES_CHECK_CUDA(cudaFuncSetAttribute(gett_tc_kernel<BN, STAGES, TC_KC, NP, false>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM));
        attr_set.fetch_or(bit);
    }
    TcArgs g = t;
    g.tiles = tiles;
    if (g.ksplit <= 1) {
        g.ksplit = 1;
        g.kper = g.kblocks;
        g.partial = nullptr;
    }
    // alpha = +-2^k, |k| <= 8, is folded into the FP32 row scale, which
    // changes only the exponent (exact); the raw split-K partials never take it
    int ak = 0;
    const double am = std::frexp(std::fabs(g.alpha), &ak);
    g.alpha_pow2 = (!g.partial && am == 0.5 && ak - 1 >= -8 && ak - 1 <= 8) ? 1 : 0;
    g.alpha_k = g.alpha_pow2 ? ak - 1 : 0;
    g.alpha_neg = (g.alpha_pow2 && g.alpha < 0) ? 1 : 0;
    g.beta_mode = g.beta == 0.0 ? 0 : (g.beta == 1.0 ? (g.Cin == g.C ? 1 : 2) : 3);
    // A ragged last round (at most a quarter of the SMs busy) has its tiles split over K so that
    // it keeps every SM busy: 2600 tiles on 152 SMs run as 17 full rounds plus 16 tiles x 9
    // parts.  With fewer parts the saving (1 - 1/parts of a round) does not cover the reduction.
    const long long sms = sm_count(ctx->device);
    g.full_items = 0;
    if (allow_tail && g.ksplit == 1) {
        const long long rounds = (tiles + sms - 1) / sms, tail = tiles - (rounds - 1) * sms;
        if (rounds >= 2 && 4 * tail <= sms && g.kblocks >= 4 * TC_KC) {
            int ks = (int)std::min<long long>(sms / tail, 16);
            int kper = (g.kblocks + ks - 1) / ks;
            kper = std::max(2 * TC_KC, (kper + TC_KC - 1) / TC_KC * TC_KC);
            ks = (g.kblocks + kper - 1) / kper;
            if (ks >= 4) {
                g.full_items = tiles - tail;
                g.tail_tiles = (int)tail;
                g.tail_ks = ks;
                g.tail_kper = kper;
                g.tail_partial = static_cast<float *>(
                    ctx->splitk_scratch((size_t)ks * tail * BN * TBM * sizeof(float)));
            }
        }
    }
    const long long items = tc_nitems(g);
    JUES_REQUIRE(items < (1LL << 31), "too many output tiles");
    // persistent: one CTA per SM (the stage ring takes most of shared memory)
    const long long grid = std::min<long long>(items, sms);
    {
        Ctx::Scope s(ctx, name);
        gett_tc_kernel<BN, STAGES, TC_KC, NP, false>
            <<<(unsigned)grid, TC_THREADS, Cfg::SMEM, ctx->stream>>>(ma, mb, g, nullptr, 0);
        JUES_CHECK_CUDA(cudaGetLastError());
    }
    if (g.full_items > 0) {
        const std::string nm = std::string(name) + ".reduce";
        Ctx::Scope s(ctx, nm.c_str());
        tail_reduce_kernel<<<dim3((unsigned)(TBM * BN / 256), (unsigned)g.tail_tiles), 256, 0, ctx->stream>>>(g, BN);
        JUES_CHECK_CUDA(cudaGetLastError());
    }
}

// Number of K splits: the wave count times the stages per split (plus a fixed per-CTA start-up
// of about five stages) is minimised over splits of at least four stages, and taken when it
// saves at least 10%: grids below two waves, and grids whose last wave is mostly empty (2.1
// waves run as 3), gain; full grids do not.  The FP32 partial sums are kept under 1 GB.
static int choose_ksplit(long long tiles, int kblocks, long long tile_elems) {
    constexpr long long kSms = 152;
    if (kblocks < 8) return 1;
    auto cost = [&](int ks) {
        const long long waves = (tiles * ks + kSms - 1) / kSms;
        return (double)waves * ((kblocks + ks - 1) / ks + 5);
    };
    int best = 1;
    for (int ks = 2; ks <= 256 && ks * 4 <= kblocks && (long long)ks * tiles * tile_elems * 4 <= (1LL << 30); ++ks)
        if (cost(ks) < cost(best)) best = ks;
    return cost(best) <= 0.9 * cost(1) ? best : 1;
}

void gett_tc(Ctx *ctx, const GettArgs &a0, const char *name, int np) {
    if (a0.M <= 0 || a0.N <= 0) return;
    JUES_REQUIRE(np == 2 || np == 3, "operand planes must be 2 or 3");
    GettArgs a = a0;
    // three planes fit TMEM and shared memory only with BN = 64
    const std::vector<int> widths = np == 3 ? std::vector<int>{64} : std::vector<int>{128, 64};
    // Orientation: the output's unit-stride mode on the row (TMEM lane) side lets each warp
    // store 32 consecutive doubles per column; weigh that against the padding of both tile
    // grids (rows pad to 128, columns to the chosen BN).
    auto pad_cost = [&](long long M, long long N, bool unit_rows) {
        long long best = -1;
        for (int cand : widths) {
            long long p = roundup(N, cand);
            if (best < 0 || p < best) best = p;
        }
        return (double)roundup(M, TBM) * (double)best * (unit_rows ? 1.0 : 1.35);
    };
    const bool m_unit = a.mC.s0 == 1 && a.mC.d0 > 1;
    const bool n_unit = a.nC.s0 == 1 && a.nC.d0 > 1;
    if (pad_cost(a.N, a.M, n_unit) < pad_cost(a.M, a.N, m_unit)) {
        std::swap(a.M, a.N);
        std::swap(a.A, a.B);
        std::swap(a.mA, a.nB);
        std::swap(a.kA, a.kB);
        std::swap(a.mC, a.nC);
        std::swap(a.a_const, a.b_const);
    }
    // skinny or tiny contractions stay in FP64
    if (a.N < 16 || a.M < 16 || a.K < 16) {
        gett_f64(ctx, a0, name);
        return;
    }
    // tile width: least padded N, a 64-wide tile weighted 1.2 (per product it moves 1.5x the
    // operand bytes of a 128-wide one, and its MMAs are half as wide), wider on ties
    int BN = widths[0];
    {
        double best = -1;
        for (int cand : widths) {
            const double p = (double)roundup(a.N, cand) * (cand == 64 && widths.size() > 1 ? 1.2 : 1.0);
            if (best < 0 || p < best) { best = p; BN = cand; }
        }
    }
    const long long Mpad = roundup(a.M, TBM), Npad = roundup(a.N, BN), Kpad = roundup(a.K, TBK);
    JUES_REQUIRE(Mpad < (1LL << 31) && Npad < (1LL << 31) && Kpad / TBK < (1LL << 30),
                 "GEMM extent exceeds the TMA coordinate range");
    const Packed pa = pack_operand(ctx, 0, a.A, a.mA, a.kA, a.M, a.K, Mpad, Kpad, a.a_const, np);
    const Packed pb = pack_operand(ctx, 1, a.B, a.nB, a.kB, a.N, a.K, Npad, Kpad, a.b_const, np);
    const CUtensorMap ma = make_map(pa.planes, Mpad, Kpad, TBM, np);
    const CUtensorMap mb = make_map(pb.planes, Npad, Kpad, BN, np);
    TcArgs t;
    t.M = a.M;
    t.N = a.N;
    t.kblocks = (int)(Kpad / TBK);
    t.mtiles = Mpad / TBM;
    t.alpha = a.alpha;
    t.beta = a.beta;
    t.C = a.C;
    t.Cin = a.Cin ? a.Cin : a.C;
    t.mC = a.mC;
    t.nC = a.nC;
    t.flags = ctx->d_flags;
    t.expA = pa.exps;
    t.expB = pb.exps;
    t.expA_ld = Mpad;
    t.expB_ld = Npad;
    const long long tiles = t.mtiles * (Npad / BN);
    JUES_REQUIRE(tiles < (1LL << 31), "too many output tiles");
    const int ks0 = choose_ksplit(tiles, t.kblocks, (long long)TBM * BN);
    if (ks0 > 1) {
        t.kper = (t.kblocks + ks0 - 1) / ks0;
        t.kper = (t.kper + TC_KC - 1) / TC_KC * TC_KC;
        t.ksplit = (t.kblocks + t.kper - 1) / t.kper;
        t.partial = static_cast<float *>(ctx->splitk_scratch((size_t)t.ksplit * Mpad * Npad * sizeof(float)));
    }
    // C = Cin + alpha AB into a dense column-major C: copy Cin over first and accumulate in
    // place, so the epilogue's adds go to L2 reductions instead of the FP64 pipe
    const bool disjoint = t.Cin + a.M * a.N <= t.C || t.C + a.M * a.N <= t.Cin;
    if (t.ksplit <= 1 && a.beta == 1.0 && t.Cin != t.C && disjoint && a.mC.d0 == MODE_BIG && a.mC.s0 == 1 &&
        a.nC.d0 == MODE_BIG && a.nC.s0 == a.M) {
        JUES_CHECK_CUDA(cudaMemcpyAsync(a.C, t.Cin, (size_t)(a.M * a.N) * sizeof(double), cudaMemcpyDeviceToDevice,
                                        ctx->stream));
        t.Cin = t.C;
    }
    if (np == 3)
        launch_tc<64, 3, 3>(ctx, ma, mb, t, tiles, name);
    else if (BN == 128)
        launch_tc<128, 3, 2>(ctx, ma, mb, t, tiles, name);
    else
        launch_tc<64, 4, 2>(ctx, ma, mb, t, tiles, name);
    if (t.ksplit > 1)
        splitk_reduce(ctx, t.partial, t.ksplit, Mpad * Npad, Mpad, a.M, a.N, a.alpha, a.beta, a.C, t.Cin, a.mC, a.nC,
                      name);
}

// ---------------------------------------------------------------------------------------
// Grouped split GEMM for the batched form: many independent GETTs, each with K <= 64, in one
// persistent launch of three-plane tcgen05 tiles.  Every problem's operand rows are packed into
// one set of planes per side (rows concatenated, one 64-wide K block), so a single tensor map
// per side covers the whole batch; the kernel finds an item's problem by binary search over the
// problems' first items.  Building (allocations, tensor maps, tables) happens once; running is
// two grouped pack launches and one GEMM launch, which a CUDA graph can capture.
// ---------------------------------------------------------------------------------------
struct TcGroup {
    std::string name;
    long long rowsA = 0, rowsB = 0, items = 0, blocksA = 0, blocksB = 0;
    std::vector<PackProb> packA, packB;
    std::vector<TcGroupProb> probs;
    DBuf<PackProb> dpackA, dpackB;
    DBuf<TcGroupProb> dprobs;
    DBuf<__half> planesA, planesB;
    DBuf<int> expA, expB;
    CUtensorMap mapA, mapB;
};

constexpr int TG_BN = 64, TG_NP = 3, TG_STAGES = 3;

TcGroup *tc_group_build(Ctx *ctx, const std::vector<GettArgs> &in, const char *name) {
    for (const GettArgs &a : in)
        if (a.K > TBK || a.K < 1) return nullptr;   // one K block per problem
    std::unique_ptr<TcGroup> tg(new TcGroup());
    tg->name = name;
    for (const GettArgs &a0 : in) {
        if (a0.M <= 0 || a0.N <= 0) continue;
        GettArgs a = a0;
        // the output's unit-stride mode on the TMEM-lane side unless padding says otherwise
        // (rows pad to 128, columns to 64)
        const bool m_unit = a.mC.s0 == 1 && a.mC.d0 > 1, n_unit = a.nC.s0 == 1 && a.nC.d0 > 1;
        const double keep = (double)roundup(a.M, TBM) * roundup(a.N, TG_BN) * (m_unit ? 1.0 : 1.35);
        const double swap = (double)roundup(a.N, TBM) * roundup(a.M, TG_BN) * (n_unit ? 1.0 : 1.35);
        if (swap < keep) {
            std::swap(a.M, a.N);
            std::swap(a.A, a.B);
            std::swap(a.mA, a.nB);
            std::swap(a.kA, a.kB);
            std::swap(a.mC, a.nC);
        }
        const long long Mpad = roundup(a.M, TBM), Npad = roundup(a.N, TG_BN);
        TcGroupProb g{};
        TcArgs &t = g.a;
        t.M = a.M;
        t.N = a.N;
        t.kblocks = 1;
        t.mtiles = Mpad / TBM;
        t.tiles = t.mtiles * (Npad / TG_BN);
        t.ksplit = 1;
        t.kper = 1;
        t.partial = nullptr;
        t.full_items = 0;
        t.alpha = a.alpha;
        t.beta = a.beta;
        int ak = 0;
        const double am = std::frexp(std::fabs(a.alpha), &ak);
        t.alpha_pow2 = (am == 0.5 && ak - 1 >= -8 && ak - 1 <= 8) ? 1 : 0;
        t.alpha_k = t.alpha_pow2 ? ak - 1 : 0;
        t.alpha_neg = (t.alpha_pow2 && a.alpha < 0) ? 1 : 0;
        t.C = a.C;
        t.Cin = a.Cin ? a.Cin : a.C;
        t.beta_mode = a.beta == 0.0 ? 0 : (a.beta == 1.0 ? (t.Cin == t.C ? 1 : 2) : 3);
        t.mC = a.mC;
        t.nC = a.nC;
        t.flags = ctx->d_flags;
        t.expA_ld = t.expB_ld = 0;   // one K chunk: the chunk stride is never used
        g.rowA = (int)tg->rowsA;
        g.rowB = (int)tg->rowsB;
        g.item0 = tg->items;
        tg->packA.push_back(PackProb{a.A, a.mA, a.kA, a.M, a.K, Mpad, tg->rowsA, tg->blocksA});
        tg->packB.push_back(PackProb{a.B, a.nB, a.kB, a.N, a.K, Npad, tg->rowsB, tg->blocksB});
        tg->rowsA += Mpad;
        tg->rowsB += Npad;
        tg->blocksA += Mpad / PR;
        tg->blocksB += Npad / PR;
        tg->items += t.tiles;
        tg->probs.push_back(g);
    }
    if (tg->probs.empty()) return tg.release();
    JUES_REQUIRE(tg->rowsA < (1LL << 31) && tg->rowsB < (1LL << 31) && tg->blocksA < (1LL << 31) &&
                     tg->blocksB < (1LL << 31) && tg->items < (1LL << 31),
                 "batch too large for one grouped launch");
    tg->planesA = DBuf<__half>(ctx, (size_t)TG_NP * tg->rowsA * TBK);
    tg->planesB = DBuf<__half>(ctx, (size_t)TG_NP * tg->rowsB * TBK);
    tg->expA = DBuf<int>(ctx, (size_t)tg->rowsA);
    tg->expB = DBuf<int>(ctx, (size_t)tg->rowsB);
    for (auto &g : tg->probs) {
        g.a.expA = tg->expA.p + g.rowA;
        g.a.expB = tg->expB.p + g.rowB;
    }
    tg->dpackA = DBuf<PackProb>(ctx, tg->packA.size());
    tg->dpackB = DBuf<PackProb>(ctx, tg->packB.size());
    tg->dprobs = DBuf<TcGroupProb>(ctx, tg->probs.size());
    JUES_CHECK_CUDA(cudaMemcpyAsync(tg->dpackA.p, tg->packA.data(), tg->packA.size() * sizeof(PackProb),
                                    cudaMemcpyHostToDevice, ctx->stream));
    JUES_CHECK_CUDA(cudaMemcpyAsync(tg->dpackB.p, tg->packB.data(), tg->packB.size() * sizeof(PackProb),
                                    cudaMemcpyHostToDevice, ctx->stream));
    JUES_CHECK_CUDA(cudaMemcpyAsync(tg->dprobs.p, tg->probs.data(), tg->probs.size() * sizeof(TcGroupProb),
                                    cudaMemcpyHostToDevice, ctx->stream));
    tg->mapA = make_map(tg->planesA.p, tg->rowsA, TBK, TBM, TG_NP);
    tg->mapB = make_map(tg->planesB.p, tg->rowsB, TBK, TG_BN, TG_NP);
    JUES_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));   // the host tables stay valid until then
    return tg.release();
}

void tc_group_run(Ctx *ctx, TcGroup *tg) {
    if (!tg || tg->probs.empty()) return;
    using Cfg = TcCfg<TG_BN, TG_STAGES, TC_KC, TG_NP>;
    {
        Ctx::Scope s(ctx, "pack_grouped");
        pack_grouped_kernel<TG_NP><<<(unsigned)tg->blocksA, 256, 0, ctx->stream>>>(
            tg->dpackA.p, (int)tg->packA.size(), tg->rowsA, tg->expA.p, tg->planesA.p);
        JUES_CHECK_CUDA(cudaGetLastError());
        pack_grouped_kernel<TG_NP><<<(unsigned)tg->blocksB, 256, 0, ctx->stream>>>(
            tg->dpackB.p, (int)tg->packB.size(), tg->rowsB, tg->expB.p, tg->planesB.p);
        ctx->count_launch();
        JUES_CHECK_CUDA(cudaGetLastError());
    }
    static std::atomic<unsigned long long> attr_set{0};
    const unsigned long long bit = ctx->device >= 0 && ctx->device < 64 ? 1ull << ctx->device : 0ull;
    if (!bit || !(attr_set.load() & bit)) {
        JUES_CHECK_CUDA(cudaFuncSetAttribute(gett_tc_kernel<TG_BN, TG_STAGES, TC_KC, TG_NP, true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM));
        attr_set.fetch_or(bit);
    }
    TcArgs g{};
    g.tiles = tg->items;
    g.flags = ctx->d_flags;
    const long long grid = std::min<long long>(tg->items, sm_count(ctx->device));
    Ctx::Scope s(ctx, tg->name.c_str());
    gett_tc_kernel<TG_BN, TG_STAGES, TC_KC, TG_NP, true><<<(unsigned)grid, TC_THREADS, Cfg::SMEM, ctx->stream>>>(
        tg->mapA, tg->mapB, g, tg->dprobs.p, (int)tg->probs.size());
    JUES_CHECK_CUDA(cudaGetLastError());
}

void tc_group_destroy(TcGroup *tg) { delete tg; }

// ---------------------------------------------------------------------------------------
// Allocation-free variant of the split GEMM (jues_gemm_noalloc).
//
// Some callers cannot let the library allocate device memory when they need a contraction:
// host frameworks that reserve the GPU's memory at start-up and hand it out from their own pool
// allocator (a cudaMalloc from inside the library would fail or escape their accounting), and
// long-running or fixed-budget services that must not grow their device footprint after
// start-up.  For them this variant packs its operands into one statically sized device array
// that is part of the loaded module (every GPU that loads the library holds it until the process
// exits) and allocates nothing itself.  The caller provides inputs and output in device memory.
// The call ends by reading the device error flags, so it is synchronous at return.
// ---------------------------------------------------------------------------------------
constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(64) << 20;   // 64 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
void *g_noalloc_addr[kMaxDevices] = {};
std::mutex g_noalloc_mutex;

// Device address of the static scratch on the current device.  Host code sees the array's
// name only as a host-side stand-in, so the address is fetched from the runtime once per
// device (with that device current) and cached.
void *noalloc_scratch_address(int device) {
    JUES_REQUIRE(device >= 0 && device < kMaxDevices, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[device]) {
        void *p = nullptr;
        JUES_CHECK_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        if (!p) throw Error(JUES_ECUDA, "cudaGetSymbolAddress returned a null scratch address");
        g_noalloc_addr[device] = p;
    }
    return g_noalloc_addr[device];
}

void pack_into(Ctx *ctx, const double *src, const Mode &rm, const Mode &km, long long R, long long K,
               long long Rpad, long long Kpad, __half *dst, int *ex) {
    Ctx::Scope s(ctx, "pack_split_noalloc");
    launch_pack<2>(ctx, src, rm, km, R, K, Rpad, Kpad, ex, dst);
}
}  // namespace

size_t gett_tc_noalloc_limit() { return NOALLOC_SCRATCH_BYTES; }

void expired_wait(Ctx *ctx) {
    {
        Ctx::Scope s(ctx, "expired_wait");
        expired_wait_kernel<<<1, 32, 0, ctx->stream>>>(ctx->d_flags);
        JUES_CHECK_CUDA(cudaGetLastError());
    }
    ctx->check_flags();   // throws JUES_ETIMEOUT and clears the flag
}

// C = beta C over an M x N output (K = 0: the product is empty); beta = 0 writes zeros
__global__ void __launch_bounds__(256) scale_output_kernel(double *C, Mode mC, Mode nC, long long M, long long N,
                                                           double beta) {
    const long long total = M * N;
    for (long long e = blockIdx.x * 256LL + threadIdx.x; e < total; e += (long long)gridDim.x * 256) {
        const long long m = e % M, n = e / M;
        double *p = C + mode_off(mC, m) + mode_off(nC, n);
        *p = beta == 0.0 ? 0.0 : beta * *p;
    }
}

// ---------------------------------------------------------------------------------------
// K-stacked operands.  Several operands with the same rows packed side by side along K into one
// buffer (each block starting on a scaling-chunk boundary) form one longer contraction:
// sum_s A_s . B_s^T is one GEMM over the stacked K, so its output tiles are written once and
// their per-tile cost is paid once.  A view reads any run of adjacent blocks.
// ---------------------------------------------------------------------------------------
void StackedPack::ensure(Ctx *ctx, long long rows, long long kcols, int planes) {
    JUES_REQUIRE(planes == 2 || planes == 3, "stacked packs hold 2 or 3 planes");
    JUES_REQUIRE(kcols % KCH == 0, "stacked pack width must be a multiple of 128");
    rows = roundup(rows, TBM);
    if (rows == rows_pad && kcols == pitch && planes == np && buf.p) return;
    buf.reset();
    exps.reset();
    rows_pad = rows;
    pitch = kcols;
    np = planes;
    buf = DBuf<uint16_t>(ctx, (size_t)np * rows_pad * pitch);
    exps = DBuf<int>(ctx, (size_t)(pitch / KCH) * rows_pad);
}

PackedView StackedPack::view(long long k0, long long kcols) const {
    JUES_REQUIRE(k0 % KCH == 0 && kcols % KCH == 0 && k0 >= 0 && k0 + kcols <= pitch, "stacked view out of range");
    PackedView v;
    v.planes = buf.p + k0;
    v.exps = exps.p + (k0 / KCH) * rows_pad;
    v.rows_pad = rows_pad;
    v.kpad = kcols;
    v.pitch = pitch;
    v.np = np;
    return v;
}

void pack_stacked(Ctx *ctx, StackedPack &sp, long long k0, const double *src, const Mode &rm, const Mode &km,
                  long long R, long long K, double scale) {
    const long long kcols = roundup(K, KCH);
    JUES_REQUIRE(R <= sp.rows_pad && k0 % KCH == 0 && k0 + kcols <= sp.pitch, "operand does not fit its stacked pack");
    int ak = 0;
    JUES_REQUIRE(std::frexp(std::fabs(scale), &ak) == 0.5, "stacked pack scale must be a power of two");
    __half *dst = reinterpret_cast<__half *>(sp.buf.p) + k0;
    int *ex = sp.exps.p + (k0 / KCH) * sp.rows_pad;
    Ctx::Scope s(ctx, "pack_split");
    if (sp.np == 3)
        launch_pack<3>(ctx, src, rm, km, R, K, sp.rows_pad, kcols, ex, dst, sp.pitch, sp.rows_pad * sp.pitch, scale);
    else
        launch_pack<2>(ctx, src, rm, km, R, K, sp.rows_pad, kcols, ex, dst, sp.pitch, sp.rows_pad * sp.pitch, scale);
}

void gett_tc_views(Ctx *ctx, const PackedView &A, const PackedView &B, long long M, long long N, double alpha,
                   double beta, double *C, const Mode &mC, const Mode &nC, const double *Cin, const char *name) {
    if (M <= 0 || N <= 0) return;
    JUES_REQUIRE(A.np == B.np && A.kpad == B.kpad, "stacked views differ in planes or K");
    JUES_REQUIRE(M <= A.rows_pad && N <= B.rows_pad, "stacked view has fewer rows than the GEMM");
    const int np = A.np;
    const int BN = (np == 2 && B.rows_pad % 128 == 0) ? 128 : 64;
    const long long Mpad = A.rows_pad, Npad = roundup(N, BN), Kpad = A.kpad;
    JUES_REQUIRE(Npad <= B.rows_pad, "stacked B view rows not a multiple of the tile width");
    const __half *pa = reinterpret_cast<const __half *>(A.planes);
    const __half *pb = reinterpret_cast<const __half *>(B.planes);
    const CUtensorMap ma = make_map(pa, A.rows_pad, Kpad, TBM, np, A.pitch);
    const CUtensorMap mb = make_map(pb, B.rows_pad, Kpad, BN, np, B.pitch);
    TcArgs t;
    t.M = M;
    t.N = N;
    t.kblocks = (int)(Kpad / TBK);
    t.mtiles = roundup(M, TBM) / TBM;
    t.alpha = alpha;
    t.beta = beta;
    t.C = C;
    t.Cin = Cin ? Cin : C;
    t.mC = mC;
    t.nC = nC;
    t.flags = ctx->d_flags;
    t.expA = A.exps;
    t.expB = B.exps;
    t.expA_ld = A.rows_pad;
    t.expB_ld = B.rows_pad;
    (void)Mpad;
    const long long tiles = t.mtiles * (Npad / BN);
    JUES_REQUIRE(tiles < (1LL << 31), "too many output tiles");
    const int ks0 = choose_ksplit(tiles, t.kblocks, (long long)TBM * BN);
    if (ks0 > 1) {
        t.kper = (t.kblocks + ks0 - 1) / ks0;
        t.kper = (t.kper + TC_KC - 1) / TC_KC * TC_KC;
        t.ksplit = (t.kblocks + t.kper - 1) / t.kper;
        t.partial = static_cast<float *>(
            ctx->splitk_scratch((size_t)t.ksplit * roundup(M, TBM) * Npad * sizeof(float)));
    }
    // C = Cin + alpha AB into a dense column-major C: copy Cin over first and accumulate in place
    const bool disjoint = t.Cin + M * N <= t.C || t.C + M * N <= t.Cin;
    if (t.ksplit <= 1 && beta == 1.0 && t.Cin != t.C && disjoint && mC.d0 == MODE_BIG && mC.s0 == 1 &&
        nC.d0 == MODE_BIG && nC.s0 == M) {
        JUES_CHECK_CUDA(cudaMemcpyAsync(C, t.Cin, (size_t)(M * N) * sizeof(double), cudaMemcpyDeviceToDevice,
                                        ctx->stream));
        t.Cin = t.C;
    }
    if (np == 3)
        launch_tc<64, 3, 3>(ctx, ma, mb, t, tiles, name);
    else if (BN == 128)
        launch_tc<128, 3, 2>(ctx, ma, mb, t, tiles, name);
    else
        launch_tc<64, 4, 2>(ctx, ma, mb, t, tiles, name);
    if (t.ksplit > 1)
        splitk_reduce(ctx, t.partial, t.ksplit, roundup(M, TBM) * Npad, roundup(M, TBM), M, N, alpha, beta, C, t.Cin,
                      mC, nC, name);
}

void gett_tc_noalloc(Ctx *ctx, const GettArgs &a) {
    if (a.M <= 0 || a.N <= 0) return;
    JUES_REQUIRE(a.K >= 0, "K must be non-negative");
    JUES_REQUIRE(!a.Cin || a.Cin == a.C, "the allocation-free GEMM accumulates into C itself");
    if (a.K == 0) {
        const long long blocks = std::min<long long>((a.M * a.N + 255) / 256, 152LL * 8);
        Ctx::Scope s(ctx, "gemm_noalloc_scale");
        scale_output_kernel<<<(unsigned)blocks, 256, 0, ctx->stream>>>(a.C, a.mC, a.nC, a.M, a.N, a.beta);
        JUES_CHECK_CUDA(cudaGetLastError());
        return;
    }
    // fixed orientation and tile width: BN = 128, the A operand on the TMEM-lane side
    constexpr int BN = 128;
    const long long Mpad = roundup(a.M, TBM), Npad = roundup(a.N, BN), Kpad = roundup(a.K, TBK);
    const long long nchunk = (Kpad + KCH - 1) / KCH;
    const size_t planesA = (size_t)2 * Mpad * Kpad * sizeof(__half);
    const size_t planesB = (size_t)2 * Npad * Kpad * sizeof(__half);
    const size_t expsA = (size_t)nchunk * Mpad * sizeof(int), expsB = (size_t)nchunk * Npad * sizeof(int);
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t need = up(planesA) + up(planesB) + up(expsA) + up(expsB);
    if (need > NOALLOC_SCRATCH_BYTES)
        throw Error(JUES_EINVAL, "jues_gemm_noalloc: this GEMM needs " + std::to_string(need) +
                                     " bytes of packed operands, more than the static scratch of " +
                                     std::to_string(NOALLOC_SCRATCH_BYTES) + " bytes");
    unsigned char *base = static_cast<unsigned char *>(noalloc_scratch_address(ctx->device));
    __half *pa = reinterpret_cast<__half *>(base);
    __half *pb = reinterpret_cast<__half *>(base + up(planesA));
    int *ea = reinterpret_cast<int *>(base + up(planesA) + up(planesB));
    int *eb = reinterpret_cast<int *>(base + up(planesA) + up(planesB) + up(expsA));
    // every byte the kernels read is rewritten here: planes including their zero padding, and
    // every (chunk,row) scale
    pack_into(ctx, a.A, a.mA, a.kA, a.M, a.K, Mpad, Kpad, pa, ea);
    pack_into(ctx, a.B, a.nB, a.kB, a.N, a.K, Npad, Kpad, pb, eb);
    const CUtensorMap ma = make_map(pa, Mpad, Kpad, TBM, 2);
    const CUtensorMap mb = make_map(pb, Npad, Kpad, BN, 2);
    TcArgs t;
    t.M = a.M;
    t.N = a.N;
    t.kblocks = (int)(Kpad / TBK);
    t.mtiles = Mpad / TBM;
    t.alpha = a.alpha;
    t.beta = a.beta;
    t.C = a.C;
    t.Cin = a.Cin ? a.Cin : a.C;
    t.mC = a.mC;
    t.nC = a.nC;
    t.flags = ctx->d_flags;
    t.expA = ea;
    t.expB = eb;
    t.expA_ld = Mpad;
    t.expB_ld = Npad;
    const long long tiles = t.mtiles * (Npad / BN);
    JUES_REQUIRE(tiles < (1LL << 31), "too many output tiles");
    launch_tc<BN, 3, 2>(ctx, ma, mb, t, tiles, "gemm_noalloc", false);   // no scratch: no tail split
}

}  // namespace jues
