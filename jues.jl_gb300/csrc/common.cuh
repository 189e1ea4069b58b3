// Shared definitions of libjuesgpu: context, errors, device buffers, tensor modes.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/jues_gpu.h"

namespace jues {

// ---------------------------------------------------------------------------------------
// errors: internal code throws jues::Error; the C ABI layer converts to a status code and
// stores the message for jues_last_error().
// ---------------------------------------------------------------------------------------
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string &msg);

#define JUES_CHECK_CUDA(expr)                                                             \
    do {                                                                                  \
        cudaError_t _e = (expr);                                                          \
        if (_e != cudaSuccess)                                                            \
            throw ::jues::Error(JUES_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(_e) + \
                                " (" __FILE__ ":" + std::to_string(__LINE__) + ")");       \
    } while (0)

#define JUES_REQUIRE(cond, msg)                                                           \
    do {                                                                                  \
        if (!(cond)) throw ::jues::Error(JUES_EINVAL, (msg));                              \
    } while (0)

// ---------------------------------------------------------------------------------------
// A tensor "mode": one GEMM dimension that is really up to three tensor indices.
// Index r maps to the element offset
//     (r % d0) * s0 + ((r / d0) % d1) * s1 + (r / (d0 * d1)) * s2.
// A plain dimension with stride s is {BIG, 1, s, 0, 0}.
// ---------------------------------------------------------------------------------------
struct Mode {
    long long d0, d1;
    long long s0, s1, s2;
};
constexpr long long MODE_BIG = (1LL << 60);
inline Mode plain(long long stride) { return Mode{MODE_BIG, 1, stride, 0, 0}; }
inline Mode mode2(long long d0, long long s0, long long s1) { return Mode{d0, MODE_BIG, s0, s1, 0}; }
inline Mode mode3(long long d0, long long d1, long long s0, long long s1, long long s2) {
    return Mode{d0, d1, s0, s1, s2};
}
// 64-bit integer division is a long instruction sequence on the GPU; plain modes need none, and
// indices and extents below 2^32 divide in 32 bits
__host__ __device__ inline void divmod_ll(long long r, long long d, long long &q, long long &rem) {
    if ((unsigned long long)r < (1ull << 32) && (unsigned long long)d < (1ull << 32)) {
        const unsigned rr = (unsigned)r, dd = (unsigned)d, qq = rr / dd;
        q = qq;
        rem = (long long)(rr - qq * dd);
    } else {
        q = r / d;
        rem = r - q * d;
    }
}
__host__ __device__ inline long long mode_off(const Mode &m, long long r) {
    if (m.d0 == MODE_BIG) return r * m.s0;
    long long q, i0;
    divmod_ll(r, m.d0, q, i0);
    if (m.d1 == MODE_BIG) return i0 * m.s0 + q * m.s1;
    long long q2, i1;
    divmod_ll(q, m.d1, q2, i1);
    return i0 * m.s0 + i1 * m.s1 + q2 * m.s2;
}

// ---------------------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------------------
struct ProfRec {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pool;
    double total_ms = 0.0;
    long long launches = 0;
};

struct PackCache;  // split-precision operand cache (gett_tc.cu)
struct BatchCache;  // batched MP2 plans and graphs (batch.cu)
struct Staging;     // page-locked staging ring and copy threads (staging.cu)

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    size_t mem_limit = 0;   // 0 = unlimited
    size_t mem_used = 0;
    bool profiling = false;
    long long launches = 0;
    std::map<std::string, ProfRec> prof;
    unsigned int *d_flags = nullptr;   // device error flags (timeouts, non-finite)
    double *d_red = nullptr;           // reduction scratch (1 << 16 doubles)
    PackCache *pack = nullptr;         // owned; destroyed by pack_cache_destroy
    BatchCache *batch = nullptr;       // owned; destroyed by batch_cache_destroy
    Staging *staging = nullptr;        // owned; destroyed by staging_destroy
    void *splitk_ws = nullptr;         // split-K partial sums, grown on demand
    size_t splitk_bytes = 0;
    cudaMemPool_t pool = nullptr;      // stream-ordered pool behind alloc/free (keeps freed memory)
    // the device reads pageable host memory through the host page tables (ATS, e.g. Grace), so
    // the split forms can pack host operands without a device copy (jues_ctx_set_ao_direct)
    bool ao_direct = false;
    bool ao_direct_supported = false;
    int batch_form = 0;   // batched form: 0 autotune, 1 FP64 tiles only, 2 tcgen05 where built
                          // (jues_ctx_set_batch_form)
    Ctx();
    ~Ctx();

    void *alloc(size_t bytes);
    void free(void *p, size_t bytes);
    void *splitk_scratch(size_t bytes);   // stream-ordered reuse: one split-K GEMM at a time
    void sync() { JUES_CHECK_CUDA(cudaStreamSynchronize(stream)); }
    // bracket a launch with profiling events when profiling is on
    struct Scope {
        Ctx *c;
        ProfRec *r = nullptr;
        std::pair<cudaEvent_t, cudaEvent_t> ev{};
        Scope(Ctx *c, const char *name);
        ~Scope();
    };
    void flush_profile();
    void count_launch() { ++launches; }
    // host wall time of a phase ("host:..." entries of the profile), recorded when profiling is
    // on; the stream is synchronised at both ends so device work is attributed to its phase
    struct HostPhase {
        Ctx *c;
        const char *name;
        double t0 = 0.0;
        HostPhase(Ctx *c, const char *name);
        ~HostPhase();
    };
    void check_flags();   // reads d_flags after a sync; throws on a set flag
};

// device buffer owned by a context
template <class T>
struct DBuf {
    Ctx *ctx = nullptr;
    T *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(Ctx *c, size_t count) : ctx(c), p(nullptr), n(count) {
        if (count) p = static_cast<T *>(c->alloc(count * sizeof(T)));
    }
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    DBuf(DBuf &&o) noexcept : ctx(o.ctx), p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DBuf &operator=(DBuf &&o) noexcept {
        reset();
        ctx = o.ctx; p = o.p; n = o.n;
        o.p = nullptr; o.n = 0;
        return *this;
    }
    ~DBuf() { reset(); }
    void reset() {
        if (p && ctx) ctx->free(p, n * sizeof(T));
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
};

// flag bits in Ctx::d_flags[0]
constexpr unsigned FLAG_TIMEOUT = 1u;
constexpr unsigned FLAG_NONFINITE = 2u;

// ---------------------------------------------------------------------------------------
// GEMM over tensor modes ("GETT"):
//   C[mC(m) + nC(n)] = alpha * sum_k A[mA(m) + kA(k)] * B[kB(k) + nB(n)] + beta * C[...]
// for m < M, n < N, k < K; beta == 0 never reads C.
// ---------------------------------------------------------------------------------------
struct GettArgs {
    long long M, N, K;
    double alpha, beta;
    const double *A; Mode mA, kA;
    const double *B; Mode kB, nB;
    double *C; Mode mC, nC;
    const double *Cin = nullptr;   // beta term reads Cin (same modes as C) when set, else C
    // split precision: operands whose values do not change between calls may be cached
    bool a_const = false, b_const = false;
};

void gett_f64(Ctx *ctx, const GettArgs &g, const char *name);
// split precision on tcgen05: np = 2 operand planes (hi, lo; JUES_PREC_SPLIT_BF16) or 3 (hi,
// mid, lo; JUES_PREC_SPLIT3)
void gett_tc(Ctx *ctx, const GettArgs &g, const char *name, int np = 2);
inline bool is_split(int precision) {
    return precision == JUES_PREC_SPLIT || precision == JUES_PREC_SPLIT3 || precision == JUES_PREC_SPLIT2;
}
inline bool valid_precision(int precision) { return precision == JUES_PREC_FP64 || is_split(precision); }
// Arithmetic of a contraction whose result is an integral (four-index transforms, get_eri blocks,
// DF factors and blocks, the MP2 adjoint's back-transforms).  Their rounding enters every energy
// directly (two planes gave MP2 -4.8e-6 Eh at nbf=200, three -2.9e-10), so the split form keeps
// three planes there; JUES_PREC_SPLIT2 keeps two.
inline int integral_precision(int precision) {
    return precision == JUES_PREC_SPLIT ? JUES_PREC_SPLIT3 : precision;
}
// split-K epilogue: C[mC(m) + nC(n)] = alpha sum_s ws[s sstride + n ld + m] + beta Cin[...],
// the partials summed in FP64 in split order (deterministic)
void splitk_reduce(Ctx *ctx, const float *ws, int ks, long long sstride, long long ld, long long M, long long N,
                   double alpha, double beta, double *C, const double *Cin, const Mode &mC, const Mode &nC,
                   const char *name);
void splitk_reduce(Ctx *ctx, const double *ws, int ks, long long sstride, long long ld, long long M, long long N,
                   double alpha, double beta, double *C, const double *Cin, const Mode &mC, const Mode &nC,
                   const char *name);
void gett(Ctx *ctx, int precision, const GettArgs &g, const char *name);
// K-stacked split-precision operands (gett_tc.cu).  A StackedPack holds np planes of rows_pad x
// pitch FP16 digits and their [chunk][row] scales; pack_stacked writes one operand (R x K over the
// modes, times a power-of-two scale) into K columns [k0, k0 + roundup(K, 128)), and a view of
// adjacent blocks is one operand of gett_tc_views, which runs C = alpha A.B^T + beta Cin over the
// stacked K.  So sum_s A_s B_s^T is one GEMM.
struct PackedView {
    const uint16_t *planes = nullptr;
    const int *exps = nullptr;
    long long rows_pad = 0, kpad = 0, pitch = 0;
    int np = 2;
};
struct StackedPack {
    DBuf<uint16_t> buf;
    DBuf<int> exps;
    long long rows_pad = 0, pitch = 0;
    int np = 2;
    void ensure(Ctx *ctx, long long rows, long long kcols, int planes);
    PackedView view(long long k0, long long kcols) const;
};
void pack_stacked(Ctx *ctx, StackedPack &sp, long long k0, const double *src, const Mode &rm, const Mode &km,
                  long long R, long long K, double scale);
void gett_tc_views(Ctx *ctx, const PackedView &A, const PackedView &B, long long M, long long N, double alpha,
                   double beta, double *C, const Mode &mC, const Mode &nC, const double *Cin, const char *name);

// Grouped three-plane split GEMM of many independent problems with K <= 64 (the batched form):
// build once (null when some problem has K > 64), then run (capturable in a CUDA graph)
struct TcGroup;
TcGroup *tc_group_build(Ctx *ctx, const std::vector<GettArgs> &probs, const char *name);
void tc_group_run(Ctx *ctx, TcGroup *g);
void tc_group_destroy(TcGroup *g);
// split GEMM that packs into a static device array instead of allocating (see gett_tc.cu)
void gett_tc_noalloc(Ctx *ctx, const GettArgs &g);
// one device wait that nothing completes: throws JUES_ETIMEOUT after the bounded wait expires
void expired_wait(Ctx *ctx);
size_t gett_tc_noalloc_limit();
void pack_cache_clear(Ctx *ctx);
void pack_cache_destroy(PackCache *p);
void batch_cache_destroy(BatchCache *p);
void batch_rmp2(Ctx *ctx, int nsys, const jues_mp2_system *sys, int precision, double e_bar, double *e_out,
                double **gao_bar, double **C_bar, jues_batch_info *info);
void pack_cache_drop(Ctx *ctx, const void *ptr);
void pack_cache_forget(Ctx *ctx, const void *p, size_t bytes);   // on every free of device memory

// ---------------------------------------------------------------------------------------
// bandwidth kernels (kernels.cu)
// ---------------------------------------------------------------------------------------
// out[mode_out(x)] = alpha * in[mode_in(x)] + beta * out[...], x over a d0*d1*d2*d3 box
// described by per-dimension strides.
struct Perm4 {
    long long d[4];
    long long si[4];
    long long so[4];
};
void permute4(Ctx *ctx, const Perm4 &p, double alpha, const double *in, double beta, double *out);
void fill(Ctx *ctx, double *p, size_t n, double v);
void axpby(Ctx *ctx, size_t n, double a, const double *x, double b, const double *y, double *out);
// sum_i x_i*y_i in FP64 (deterministic two-pass block reduction)
double dot(Ctx *ctx, size_t n, const double *x, const double *y);
// MP2: sum K[i,j,a,b](2K[i,j,a,b]-K[i,j,b,a]) / D (K column-major [i,j,a,b])
double mp2_energy(Ctx *ctx, const double *K, const double *eps, int o, int v);
// MP2 adjoint seed: G[i,a,j,b] = 2 e_bar (2K[i,a,j,b] - K[i,b,j,a]) / D from chemists' K (G may be
// null: energy only); returns E
double mp2_gamma(Ctx *ctx, const double *K, const double *eps, int o, int v, double e_bar, double *G);
// CC energy: sum oovv[i,j,a,b] (2 X[i,j,a,b] - X[j,i,a,b]) with X = T2 (+ t1 t1 when t1)
double cc_energy(Ctx *ctx, const double *oovv, const double *T2, const double *t1, int o, int v);
// T2 finalisation: Tn[i,j,a,b] = (L + Z[i,j,a,b] + Z[j,i,b,a] + C[i,j,a,b] + C[j,i,b,a]) invD
// with C[i,j,a,b] = t1[i,a] q[b,j] when t1 and q (v x o) are given; returns ||Tn - Told||^2 if
// Told != nullptr.  Writes Tn.
// with pairl, L = [L+ | L-] (the folded ladders) and invD the folded 1/D (inv_denominators_folded)
double t2_finalize(Ctx *ctx, const double *L, const double *Z, const double *invD, int o, int v,
                   const double *Told, double *Tn, const double *t1 = nullptr, const double *q = nullptr,
                   bool pairl = false);
// whether t2_finalize takes folded ladders (pairl) at these sizes
bool t2_finalize_folds(int o, int v);
// folding of a pair-symmetric contraction over an index pair (e <= f) of extent d (kernels.cu,
// pair_fold_kernel): out = [out+ | out-], each R x d(d+1)/2
void pair_fold(Ctx *ctx, const double *src, long long R, bool rowpair, long long rd, long long rs0, long long rs1,
               int d, long long ke, long long kf, double scale, bool diag_half, double *out);
// the inverse over an occupied pair (i <= j) (pair_unfold_kernel)
void pair_unfold(Ctx *ctx, const double *P, long long npc, const double *base, int o, long long C, long long sij,
                 long long sc, long long tp, long long tc, bool ijfast, double *out);
// invD[i,j,a,b] = 1 / (e_i + e_j - e_a - e_b)
void inv_denominators(Ctx *ctx, const double *eps, int o, int v, double *out);
// the same over occupied pairs p = (i <= j) and virtual pairs q = (a <= b): out[p + np q]
void inv_denominators_folded(Ctx *ctx, const double *eps, int o, int v, double *out);
// t1n[i,a] /= (e_i - e_a) in place; returns ||t1n - t1old||^2
double t1_finalize(Ctx *ctx, double *t1n, const double *eps, int o, int v, const double *t1old);
// X[i,j,a,b] = (L[...]) / D in place variants used for guesses
void divide_by_d(Ctx *ctx, const double *in, const double *eps, int o, int v, double *out);
// T~ = 2 T[i,j,a,b] - T[j,i,a,b]
void t_tilde(Ctx *ctx, const double *T, int o, int v, double *out);
// sum_k c_k * vecs[k] -> out (length n)
void lincomb(Ctx *ctx, size_t n, int m, const double *const *vecs, const double *c, double *out);
// W'[(m,n),(i,j)] -= [m = i] Fmi[n,j] + [n = j] Fmi[m,i] (o^4 W', o x o Fmi, column-major)
void wp_fmi(Ctx *ctx, double *Wp, const double *Fmi, int o);
// Fmi[m,i] = sum_n 2 X[m,n,i,n] - X[m,n,n,i], X = Wp - oooo (o^4 arrays [(m,n),(i,j)])
void fmi_from_x(Ctx *ctx, const double *Wp, const double *oooo, int o, double *Fmi);
// Fae[a,e] = -(cJ (tr WJ - trJ0) + cK (tr WK - trK0))[a,e], traces over m of [(m,e),(a,m)] (trJ0, trK0:
// the seeds' traces); when W12 is given, W12[(j,e),(a,j)] += Fae[a,e] for every j
void fae_from_rings(Ctx *ctx, const double *WJ, const double *trJ0, const double *WK, const double *trK0, int o,
                    int v, double cJ, double cK, double *Fae, double *W12);
// CCSD: Ttau = T2 + t1 (x) t1 and U = T2 + 2 t1 (x) t1
void ccsd_tau(Ctx *ctx, const double *T, const double *t1, int o, int v, double *Ttau, double *U);
// traces over m of WJ and WK at [(m,e),(a,m)] less trJ0, trK0 (null: nothing) into tJ[a,e], tK[a,e]
void ring_traces(Ctx *ctx, const double *WJ, const double *trJ0, const double *WK, const double *trK0, int o, int v,
                 double *tJ, double *tK);
// CCSD Fae, H1, G2 from the ring traces, and F~ae onto W12's (m = j) entries (kernels.cu)
void ccsd_fae(Ctx *ctx, const double *WJ, const double *trJ0, const double *WK, const double *trK0, const double *tGJ,
              const double *tGK, const double *t1, const double *c12, const double *Fme, const double *fOV,
              const double *fVV, int o, int v, bool mvariant, double *Fae, double *H1, double *G2, double *W12);
// R1 += T1's <ma|fe> terms from the traces of Y[(i,j),(a,m)], which carries the ooov seed
// ooov[m,i,j,a] (its traces c2, c3 from c123 are taken off)
void t1_ytrace(Ctx *ctx, const double *Y, const double *t1, const double *G2, const double *H1, const double *c123,
               int o, int v, double *R1);
// R1[i,a] += sum_{m,e} (2 T2[i,m,a,e] - T2[m,i,a,e]) Fme[m,e] (one read of T2; o <= 64)
void t1_fme(Ctx *ctx, const double *T, const double *Fme, int o, int v, double *R1);
// c1[n,e] = sum_m ooov[n,m,m,e], c2[n,e] = sum_m ooov[m,n,m,e], c3[n,e] = sum_m ooov[m,m,n,e] into
// c12[0..ov), [ov..2ov), [2ov..3ov)
void ooov_diag_sums(Ctx *ctx, const double *ooov, int o, int v, double *c12);
// DIIS bookkeeping in one pass: v_out = xn (skipped when null), e_out = xn - x, dots[0] = e.e,
// dots[1 + k] = olds[k].e
void diis_error(Ctx *ctx, size_t n, const double *xn, const double *x, double *v_out, double *e_out, int nold,
                const double *const *olds, double *dots);
// 1 if any element of x is NaN/Inf
bool any_nonfinite(Ctx *ctx, const double *x, size_t n);

}  // namespace jues

struct jues_ctx {
    jues::Ctx impl;
};
