// extern "C" entry points of libjuesgpu.so (declared in include/jues_gpu.h).
#include <algorithm>
#include <cstdlib>
#include <chrono>
#include <cstring>
#include <string>

#include "cc.cuh"
#include "df.cuh"
#include "fock.cuh"
#include "triples.cuh"
#include "common.cuh"
#include "transform.cuh"

using namespace jues;

namespace jues {
const std::string &last_error();
}

namespace {

template <class F>
int guarded(F &&f) {
    try {
        f();
        return JUES_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc &) {
        set_last_error("host allocation failed");
        return JUES_ENOMEM;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return JUES_EINVAL;
    }
}

Ctx &CX(jues_ctx *c) {
    if (!c) throw Error(JUES_EINVAL, "null context");
    return c->impl;
}

void need(const void *p, const char *what) {
    if (!p) throw Error(JUES_EINVAL, std::string("null pointer: ") + what);
}

// copy a host array to a new context buffer
// The AO integrals of a transform in precision prec.  Where the device reads pageable host
// memory through the host page tables, the split forms pack them straight from the caller's
// array (one pass over the NVLink-C2C link, no n^4 device copy); otherwise they are copied.
static const double *ao_operand(Ctx &c, const double *gao, size_t n4, int prec, DBuf<double> &hold);

// Host -> device copy of a caller's array.  Large pageable arrays are registered (page-locked)
// for the duration of the copy: the DMA engines then read them directly at link speed, where an
// unregistered copy is staged through the driver's bounce buffers (measured on GB300 with Grace:
// ~200 GB/s against ~6 GB/s for the 12.8 GB AO integrals at nbf=200).  Registration costs tens
// to hundreds of milliseconds for 12.8 GB, varying with the host's page state, so the array goes
// in 512 MB pieces: the next piece is registered while the link copies this one, and each piece
// is released once its copy has finished.
namespace {
struct H2DPieces {
    struct Piece {
        uintptr_t a, b;
        bool reg = false;
        cudaEvent_t done = nullptr;
    };
    Ctx &ctx;
    std::vector<Piece> ps;
    double reg_ms = 0.0, unreg_ms = 0.0;
    explicit H2DPieces(Ctx &c) : ctx(c) {}
    static double now_ms() {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
    }
    void reg(Piece &p) {
        const double t = now_ms();
        const cudaError_t e = cudaHostRegister(reinterpret_cast<void *>(p.a), p.b - p.a, cudaHostRegisterDefault);
        reg_ms += now_ms() - t;
        if (e == cudaSuccess) {
            p.reg = true;
        } else {
            cudaGetLastError();   // already page-locked by the caller, or not registrable: plain copy
            if (ctx.profiling) ctx.prof["host:register_failed_" + std::to_string((int)e)].launches += 1;
        }
    }
    void release(Piece &p) {
        if (p.done) cudaEventSynchronize(p.done);
        if (p.reg) {
            const double t = now_ms();
            cudaHostUnregister(reinterpret_cast<void *>(p.a));
            unreg_ms += now_ms() - t;
            p.reg = false;
        }
    }
    ~H2DPieces() {   // also on an error path: no range stays registered, no event leaks
        for (Piece &p : ps) {
            release(p);
            if (p.done) cudaEventDestroy(p.done);
        }
        if (ctx.profiling) {
            ctx.prof["h2d:register"].total_ms += reg_ms;
            ctx.prof["h2d:unregister"].total_ms += unreg_ms;
        }
    }
};
}  // namespace

DBuf<double> h2d(Ctx &ctx, const double *h, size_t n) {
    DBuf<double> d(&ctx, n);
    if (!n) return d;
    const size_t bytes = n * sizeof(double);
    if (bytes < (size_t(64) << 20)) {
        JUES_CHECK_CUDA(cudaMemcpyAsync(d.p, h, bytes, cudaMemcpyHostToDevice, ctx.stream));
        return d;
    }
    constexpr uintptr_t kPiece = uintptr_t(512) << 20, kAlign = uintptr_t(2) << 20;
    const uintptr_t b0 = reinterpret_cast<uintptr_t>(h), b1 = b0 + bytes;
    H2DPieces pc(ctx);
    // interior cuts on 2 MB host addresses: no two pieces share a page
    for (uintptr_t a = b0, c = (b0 + kPiece) / kAlign * kAlign; a < b1; a = c, c += kPiece) {
        const uintptr_t e = c < b1 ? c : b1;
        pc.ps.push_back({a, e});
    }
    for (auto &p : pc.ps) JUES_CHECK_CUDA(cudaEventCreateWithFlags(&p.done, cudaEventDisableTiming));
    pc.reg(pc.ps[0]);
    for (size_t i = 0; i < pc.ps.size(); ++i) {
        H2DPieces::Piece &p = pc.ps[i];
        JUES_CHECK_CUDA(cudaMemcpyAsync(d.p + (p.a - b0) / sizeof(double), reinterpret_cast<const void *>(p.a),
                                        p.b - p.a, cudaMemcpyHostToDevice, ctx.stream));
        JUES_CHECK_CUDA(cudaEventRecord(p.done, ctx.stream));
        if (i + 1 < pc.ps.size()) pc.reg(pc.ps[i + 1]);
        if (i >= 1) pc.release(pc.ps[i - 1]);
    }
    pc.release(pc.ps.back());
    return d;
}

static const double *ao_operand(Ctx &c, const double *gao, size_t n4, int prec, DBuf<double> &hold) {
    if (is_split(prec) && c.ao_direct) return gao;
    Ctx::HostPhase ph(&c, "host:h2d_ao_eri");
    hold = h2d(c, gao, n4);
    return hold.p;
}

void d2h(Ctx &ctx, double *h, const double *d, size_t n) {
    if (n) JUES_CHECK_CUDA(cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
}

void check_dims(int n, int o, int v) {
    if (n <= 0) throw Error(JUES_EINVAL, "nbf must be positive");
    if (o <= 0 || v <= 0) throw Error(JUES_EINVAL, "nocc and nvir must be positive");
    if (o + v > n) throw Error(JUES_EINVAL, "nocc + nvir exceeds nbf");
}

void check_opts(const jues_cc_opts &o) {
    if (o.maxit < 0) throw Error(JUES_EINVAL, "maxit must be >= 0");
    if (o.diis && (o.diis_size < 2 || o.diis_size > 16)) throw Error(JUES_EINVAL, "diis_size must be in 2..16");
    if (!valid_precision(o.precision))
        throw Error(JUES_EINVAL, "unknown precision");
    if (o.guess < 0 || o.guess > 2) throw Error(JUES_EINVAL, "unknown guess");
    if (o.refine < 0) throw Error(JUES_EINVAL, "refine must be >= 0");
    if (o.transform_precision != -1 && !valid_precision(o.transform_precision))
        throw Error(JUES_EINVAL, "unknown transform_precision");
    if (o.ccsd_fae != JUES_CCSD_FAE_RCCSD && o.ccsd_fae != JUES_CCSD_FAE_MRCCSD)
        throw Error(JUES_EINVAL, "unknown ccsd_fae variant");
}

}  // namespace

struct jues_cc {
    CCState *s = nullptr;
    ~jues_cc() { delete s; }
};

// the fitted factor b = pqP Jpqh on the device (pqP itself when Jpqh is null), DF.jl:52-57
static DBuf<double> fitted_factor(Ctx &c, const double *pqP, int pqP_is_device, int n, int naux,
                                  const double *Jpqh, int precision) {
    const size_t nb = (size_t)n * n * naux;
    DBuf<double> host_copy;
    const double *src = pqP;
    if (!pqP_is_device) {
        host_copy = h2d(c, pqP, nb);
        src = host_copy.p;
    }
    if (Jpqh) {
        DBuf<double> dj = h2d(c, Jpqh, (size_t)naux * naux);
        return df_fit(&c, precision, src, n, naux, dj.p);
    }
    if (!pqP_is_device) return host_copy;
    DBuf<double> b(&c, nb);
    JUES_CHECK_CUDA(cudaMemcpyAsync(b.p, pqP, nb * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
    return b;
}

extern "C" {

int jues_version(void) { return 10000; }

int jues_last_error(char *buf, size_t len) {
    if (!buf || !len) return JUES_EINVAL;
    const std::string &m = last_error();
    size_t k = m.size() < len - 1 ? m.size() : len - 1;
    std::memcpy(buf, m.data(), k);
    buf[k] = 0;
    return JUES_OK;
}

int jues_ctx_create(int device, jues_ctx **out) {
    return guarded([&] {
        need(out, "out");
        *out = nullptr;
        int ndev = 0;
        cudaError_t e = cudaGetDeviceCount(&ndev);
        if (e != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            throw Error(JUES_ENODEV, "no CUDA device available");
        }
        if (device < 0 || device >= ndev) throw Error(JUES_EINVAL, "device index out of range");
        cudaDeviceProp prop;
        JUES_CHECK_CUDA(cudaGetDeviceProperties(&prop, device));
        if (prop.major != 10 || prop.minor != 3)
            throw Error(JUES_ENODEV, std::string("libjuesgpu is built for sm_103 (GB300); device is ") +
                                         prop.name + " sm_" + std::to_string(prop.major) +
                                         std::to_string(prop.minor));
        JUES_CHECK_CUDA(cudaSetDevice(device));
        std::unique_ptr<jues_ctx> c(new jues_ctx());
        Ctx &x = c->impl;
        x.device = device;
        JUES_CHECK_CUDA(cudaStreamCreateWithFlags(&x.stream, cudaStreamNonBlocking));
        JUES_CHECK_CUDA(cudaMalloc(&x.d_flags, 4 * sizeof(unsigned)));
        JUES_CHECK_CUDA(cudaMemset(x.d_flags, 0, 4 * sizeof(unsigned)));
        JUES_CHECK_CUDA(cudaMalloc(&x.d_red, 65536 * sizeof(double)));
        int pageable = 0, host_tables = 0;
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) pageable = 0;
        if (cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) !=
            cudaSuccess)
            host_tables = 0;
        cudaGetLastError();
        const char *env = std::getenv("JUES_AO_DIRECT");
        x.ao_direct_supported = pageable == 1 && host_tables == 1;
        // off by default: reading pageable memory through the host page tables measured ~8 GB/s
        // for the AO integrals, slower than the registered copy
        x.ao_direct = x.ao_direct_supported && env && env[0] == '1';
        *out = c.release();
    });
}

int jues_ctx_set_ao_direct(jues_ctx *ctx, int enable, int *active) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        c.ao_direct = enable && c.ao_direct_supported;
        if (active) *active = c.ao_direct ? 1 : 0;
    });
}

int jues_ctx_destroy(jues_ctx *ctx) {
    return guarded([&] {
        need(ctx, "ctx");
        cudaSetDevice(ctx->impl.device);
        delete ctx;
    });
}

int jues_ctx_set_mem_limit(jues_ctx *ctx, size_t bytes) {
    return guarded([&] { CX(ctx).mem_limit = bytes; });
}

int jues_ctx_set_profiling(jues_ctx *ctx, int on) {
    return guarded([&] { CX(ctx).profiling = on != 0; });
}

int jues_ctx_profile(jues_ctx *ctx, const char *prefix, double *total_ms, long long *launches) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        need(prefix, "prefix");
        c.flush_profile();
        double t = 0.0;
        long long n = 0;
        size_t lp = std::strlen(prefix);
        for (auto &kv : c.prof) {
            if (kv.first.compare(0, lp, prefix) == 0) {
                t += kv.second.total_ms;
                n += kv.second.launches;
            }
        }
        if (total_ms) *total_ms = t;
        if (launches) *launches = n;
    });
}

int jues_ctx_profile_reset(jues_ctx *ctx) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        c.flush_profile();
        for (auto &kv : c.prof) {
            kv.second.total_ms = 0.0;
            kv.second.launches = 0;
        }
    });
}

long long jues_ctx_launch_count(jues_ctx *ctx) { return ctx ? ctx->impl.launches : -1; }

int jues_gemm(jues_ctx *ctx, int transA, int transB, int M, int N, int K, double alpha, const double *A,
              int lda, const double *B, int ldb, double beta, double *C, int ldc, int precision) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        need(A, "A"); need(B, "B"); need(C, "C");
        if (M < 0 || N < 0 || K < 0) throw Error(JUES_EINVAL, "negative GEMM dimension");
        const int ar = transA ? K : M, br = transB ? N : K;
        if (lda < std::max(1, ar) || ldb < std::max(1, br) || ldc < std::max(1, M))
            throw Error(JUES_EINVAL, "leading dimension too small");
        if (!valid_precision(precision))
            throw Error(JUES_EINVAL, "unknown precision");
        if (M == 0 || N == 0) return;
        cudaSetDevice(c.device);
        const size_t na = (size_t)lda * (transA ? M : K), nb = (size_t)ldb * (transB ? K : N),
                     nc = (size_t)ldc * N;
        DBuf<double> dA = h2d(c, A, na), dB = h2d(c, B, nb), dC = h2d(c, C, nc);
        GettArgs g;
        g.M = M; g.N = N; g.K = K;
        g.alpha = alpha; g.beta = beta;
        g.A = dA.p; g.mA = transA ? plain(lda) : plain(1); g.kA = transA ? plain(1) : plain(lda);
        g.B = dB.p; g.kB = transB ? plain(ldb) : plain(1); g.nB = transB ? plain(1) : plain(ldb);
        g.C = dC.p; g.mC = plain(1); g.nC = plain(ldc);
        gett(&c, precision, g, "gemm");
        d2h(c, C, dC.p, nc);
        c.check_flags();
    });
}

int jues_gemm_noalloc(jues_ctx *ctx, int transA, int transB, int M, int N, int K, double alpha,
                      const double *A_dev, int lda, const double *B_dev, int ldb, double beta, double *C_dev,
                      int ldc) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        need(A_dev, "A"); need(B_dev, "B"); need(C_dev, "C");
        if (M < 0 || N < 0 || K < 0) throw Error(JUES_EINVAL, "negative GEMM dimension");
        const int ar = transA ? K : M, br = transB ? N : K;
        if (lda < std::max(1, ar) || ldb < std::max(1, br) || ldc < std::max(1, M))
            throw Error(JUES_EINVAL, "leading dimension too small");
        if (M == 0 || N == 0) return;
        JUES_CHECK_CUDA(cudaSetDevice(c.device));
        GettArgs g;
        g.M = M; g.N = N; g.K = K;
        g.alpha = alpha; g.beta = beta;
        g.A = A_dev; g.mA = transA ? plain(lda) : plain(1); g.kA = transA ? plain(1) : plain(lda);
        g.B = B_dev; g.kB = transB ? plain(ldb) : plain(1); g.nB = transB ? plain(1) : plain(ldb);
        g.C = C_dev; g.mC = plain(1); g.nC = plain(ldc);
        gett_tc_noalloc(&c, g);
        c.check_flags();
    });
}

int jues_debug_expired_wait(jues_ctx *ctx) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        JUES_CHECK_CUDA(cudaSetDevice(c.device));
        expired_wait(&c);
    });
}

int jues_tei_transform(jues_ctx *ctx, const double *gao, int n, const double *C1, int d1, const double *C2,
                       int d2, const double *C3, int d3, const double *C4, int d4, int precision,
                       double *out) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        need(gao, "gao");
        need(C1, "C1"); need(C2, "C2"); need(C3, "C3"); need(C4, "C4");
        need(out, "out");
        if (n <= 0) throw Error(JUES_EINVAL, "nbf must be positive");
        if (d1 < 0 || d2 < 0 || d3 < 0 || d4 < 0) throw Error(JUES_EINVAL, "negative MO dimension");
        if (!valid_precision(precision))
            throw Error(JUES_EINVAL, "unknown precision");
        cudaSetDevice(c.device);
        const size_t n4 = (size_t)n * n * n * n;
        DBuf<double> g;
        const double *gp = ao_operand(c, gao, n4, precision, g);
        DBuf<double> c1 = h2d(c, C1, (size_t)n * d1), c2 = h2d(c, C2, (size_t)n * d2),
                     c3 = h2d(c, C3, (size_t)n * d3), c4 = h2d(c, C4, (size_t)n * d4);
        const size_t no = (size_t)d1 * d2 * d3 * d4;
        DBuf<double> dout(&c, no);
        const double *Cs[4] = {c1.p, c2.p, c3.p, c4.p};
        int d[4] = {d1, d2, d3, d4};
        long long ostr[4] = {1, d1, (long long)d1 * d2, (long long)d1 * d2 * d3};
        transform4(&c, precision, gp, n, Cs, d, dout.p, ostr, false);
        d2h(c, out, dout.p, no);
        c.check_flags();
    });
}

int jues_get_eri(jues_ctx *ctx, const double *gao, int n, const double *Cocc, int o, const double *Cvir, int v,
                 const char *spec, int phys, int fcn, int precision, double *out) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        need(gao, "gao"); need(Cocc, "Cocc"); need(Cvir, "Cvir"); need(spec, "spec"); need(out, "out");
        if (std::strlen(spec) != 4)
            throw Error(JUES_EINVAL, std::string("Invalid string given to get_eri: ") + spec);
        check_dims(n, o, v);
        if (!valid_precision(precision))
            throw Error(JUES_EINVAL, "unknown precision");
        size_t no = 1;
        for (int q = 0; q < 4; ++q) {
            char ch = spec[q];
            if (ch == 'o' || ch == 'O') {
                if (fcn < 0 || fcn > o) throw Error(JUES_EINVAL, "fcn out of range");
                no *= (size_t)(o - fcn);
            } else if (ch == 'v' || ch == 'V') {
                no *= (size_t)v;
            } else {
                throw Error(JUES_EINVAL, std::string("Invalid string given to get_eri: ") + spec);
            }
        }
        cudaSetDevice(c.device);
        DBuf<double> g;
        const double *gp = ao_operand(c, gao, (size_t)n * n * n * n, precision, g);
        DBuf<double> co = h2d(c, Cocc, (size_t)n * o), cv = h2d(c, Cvir, (size_t)n * v);
        DBuf<double> dout(&c, no);
        get_eri_block(&c, precision, gp, n, co.p, o, cv.p, v, spec, phys != 0, fcn, dout.p, false);
        d2h(c, out, dout.p, no);
        c.check_flags();
    });
}

int jues_rmp2(jues_ctx *ctx, const double *gao, int n, const double *Cocc, int o, const double *Cvir, int v,
              const double *eps, int precision, double *e_out, double *k_out) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        need(gao, "gao"); need(Cocc, "Cocc"); need(Cvir, "Cvir"); need(eps, "eps"); need(e_out, "e_out");
        check_dims(n, o, v);
        if (!valid_precision(precision))
            throw Error(JUES_EINVAL, "unknown precision");
        cudaSetDevice(c.device);
        DBuf<double> g;
        const double *gp = ao_operand(c, gao, (size_t)n * n * n * n, precision, g);
        DBuf<double> co = h2d(c, Cocc, (size_t)n * o), cv = h2d(c, Cvir, (size_t)n * v);
        DBuf<double> de = h2d(c, eps, (size_t)n);
        const size_t nk = (size_t)o * o * v * v;
        DBuf<double> K(&c, nk);
        get_eri_block(&c, precision, gp, n, co.p, o, cv.p, v, "OOVV", true, 0, K.p, false);
        g.reset();
        *e_out = mp2_energy(&c, K.p, de.p, o, v);
        if (k_out) d2h(c, k_out, K.p, nk);
        c.check_flags();
    });
}

int jues_df_rmp2(jues_ctx *ctx, const double *pqP, int n, int naux, const double *Jpqh, const double *Cocc,
                 int o, const double *Cvir, int v, const double *eps, int precision, double *e_out) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        need(pqP, "pqP"); need(Cocc, "Cocc"); need(Cvir, "Cvir"); need(eps, "eps"); need(e_out, "e_out");
        check_dims(n, o, v);
        if (naux <= 0) throw Error(JUES_EINVAL, "naux must be positive");
        if (!valid_precision(precision))
            throw Error(JUES_EINVAL, "unknown precision");
        cudaSetDevice(c.device);
        const long long ov = (long long)o * v;
        DBuf<double> b = fitted_factor(c, pqP, 0, n, naux, Jpqh, precision);
        DBuf<double> co = h2d(c, Cocc, (size_t)n * o), cv = h2d(c, Cvir, (size_t)n * v);
        DBuf<double> de = h2d(c, eps, (size_t)n);
        // B[i,a,Q] = sum_{mu,nu} Cocc[mu,i] b[mu,nu,Q] Cvir[nu,a]   (DF-RMP2.jl:17-22)
        DBuf<double> bia(&c, (size_t)(ov * naux));
        df_mo_factor(&c, precision, b.p, n, naux, co.p, o, cv.p, v, bia.p);
        b.reset();
        // (ia|jb) = sum_Q B[(ia),Q] B[(jb),Q], chemists' [i,a,j,b]   (DF-RMP2.jl:28-34)
        DBuf<double> K(&c, (size_t)(ov * ov));
        {
            GettArgs a;
            a.M = ov; a.N = ov; a.K = naux;
            a.alpha = 1.0; a.beta = 0.0;
            a.A = bia.p; a.mA = plain(1); a.kA = plain(ov);
            a.B = bia.p; a.kB = plain(ov); a.nB = plain(1);
            a.C = K.p; a.mC = plain(1); a.nC = plain(ov);
            gett(&c, integral_precision(precision), a, "df_iajb");
        }
        *e_out = mp2_gamma(&c, K.p, de.p, o, v, 1.0, nullptr);   // DF-RMP2.jl:36-42
        c.check_flags();
    });
}

int jues_rmp2_adjoint(jues_ctx *ctx, const double *gao, int n, const double *C, int o, const double *eps,
                      int precision, double e_bar, double *e_out, double *gao_bar, double *C_bar) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        need(gao, "gao"); need(C, "C"); need(eps, "eps"); need(e_out, "e_out");
        const int v = n - o;
        check_dims(n, o, v);
        if (!valid_precision(precision))
            throw Error(JUES_EINVAL, "unknown precision");
        cudaSetDevice(c.device);
        DBuf<double> gbuf;
        const double *gp = ao_operand(c, gao, (size_t)n * n * n * n, precision, gbuf);
        DBuf<double> dC = h2d(c, C, (size_t)n * n);
        DBuf<double> de = h2d(c, eps, (size_t)n);
        const double *Co = dC.p, *Cv = dC.p + (size_t)n * o;
        const long long ov = (long long)o * v;
        const size_t nk = (size_t)(ov * ov);
        // K = (ia|jb) in chemists' order
        DBuf<double> K(&c, nk), G(&c, nk);
        {
            const double *Cs[4] = {Co, Cv, Co, Cv};
            int d[4] = {o, v, o, v};
            long long ostr[4] = {1, o, ov, ov * o};
            transform4(&c, precision, gp, n, Cs, d, K.p, ostr, true);
        }
        *e_out = mp2_gamma(&c, K.p, de.p, o, v, e_bar, G.p);
        K.reset();
        if (gao_bar) {
            const double *Cs[4] = {Co, Cv, Co, Cv};
            int d[4] = {o, v, o, v};
            DBuf<double> gb(&c, (size_t)n * n * n * n);
            backtransform4(&c, precision, G.p, d, n, Cs, gb.p);
            d2h(c, gao_bar, gb.p, gb.n);
        }
        if (C_bar) {
            DBuf<double> cb(&c, (size_t)n * n);
            {
                // H[mu,a,j,b] = (mu a|j b); dE/dC[mu,i] = 2 sum_{ajb} H[mu,(ajb)] G[i,(ajb)]
                const double *Cs[4] = {nullptr, Cv, Co, Cv};
                int d[4] = {n, v, o, v};
                long long ostr[4] = {1, n, (long long)n * v, (long long)n * v * o};
                DBuf<double> H(&c, (size_t)n * v * o * v);
                transform4(&c, precision, gp, n, Cs, d, H.p, ostr, true);
                GettArgs a;
                a.M = n; a.N = o; a.K = ov * v;
                a.alpha = 2.0; a.beta = 0.0;
                a.A = H.p; a.mA = plain(1); a.kA = plain(n);
                a.B = G.p; a.kB = plain(o); a.nB = plain(1);
                a.C = cb.p; a.mC = plain(1); a.nC = plain(n);
                gett(&c, integral_precision(precision), a, "adjoint_cocc");
            }
            {
                // H'[i,nu,j,b] = (i nu|j b); dE/dC[nu,a] = 2 sum_{ijb} H'[i,nu,j,b] G[i,a,j,b]
                const double *Cs[4] = {Co, nullptr, Co, Cv};
                int d[4] = {o, n, o, v};
                long long ostr[4] = {1, o, (long long)o * n, (long long)o * n * o};
                DBuf<double> H(&c, (size_t)o * n * o * v);
                transform4(&c, precision, gp, n, Cs, d, H.p, ostr, true);
                GettArgs a;
                a.M = n; a.N = v; a.K = (long long)o * o * v;
                a.alpha = 2.0; a.beta = 0.0;
                a.A = H.p; a.mA = plain(o); a.kA = mode3(o, o, 1, (long long)o * n, (long long)o * n * o);
                a.B = G.p; a.kB = mode3(o, o, 1, ov, ov * o); a.nB = plain(o);
                a.C = cb.p + (size_t)n * o; a.mC = plain(1); a.nC = plain(n);
                gett(&c, integral_precision(precision), a, "adjoint_cvir");
            }
            d2h(c, C_bar, cb.p, cb.n);
        }
        pack_cache_drop(&c, gp);
        c.check_flags();
    });
}

int jues_ctx_set_batch_form(jues_ctx *ctx, int form) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        if (form < 0 || form > 2) throw Error(JUES_EINVAL, "batch form must be 0, 1 or 2");
        c.batch_form = form;
    });
}

int jues_batch_rmp2(jues_ctx *ctx, int nsys, const jues_mp2_system *systems, int precision, double e_bar,
                    double *e_out, double **gao_bar, double **C_bar, jues_batch_info *info) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        need(systems, "systems");
        need(e_out, "e_out");
        cudaSetDevice(c.device);
        batch_rmp2(&c, nsys, systems, precision, e_bar, e_out, gao_bar, C_bar, info);
    });
}

int jues_cc_default_opts(jues_cc_opts *opts) {
    return guarded([&] {
        need(opts, "opts");
        opts->maxit = 40;        // mRCCD.jl:38
        opts->e_conv = 0.0;
        opts->r_conv = 1e-7;     // mRCCD.jl:106
        opts->diis = 1;          // mRCCD.jl:39
        opts->diis_size = 6;     // mRCCD.jl:67
        opts->precision = JUES_PREC_FP64;
        opts->guess = JUES_GUESS_ZERO;   // mRCCD.jl:245
        opts->refine = 2;
        opts->transform_precision = -1;
        opts->ccsd_fae = JUES_CCSD_FAE_RCCSD;
    });
}

int jues_cc_create(jues_ctx *ctx, int method, const double *gao, int gao_is_device, int n, const double *Cocc,
                   int o, const double *Cvir, int v, const double *eps, const jues_cc_opts *opts,
                   jues_cc **out) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        need(gao, "gao"); need(Cocc, "Cocc"); need(Cvir, "Cvir"); need(eps, "eps"); need(out, "out");
        *out = nullptr;
        check_dims(n, o, v);
        jues_cc_opts op;
        if (opts) op = *opts; else jues_cc_default_opts(&op);
        check_opts(op);
        cudaSetDevice(c.device);
        DBuf<double> g;
        const double *gp = gao;
        if (!gao_is_device)
            gp = ao_operand(c, gao, (size_t)n * n * n * n,
                            op.transform_precision >= 0 ? op.transform_precision : op.precision, g);
        DBuf<double> co = h2d(c, Cocc, (size_t)n * o), cv = h2d(c, Cvir, (size_t)n * v);
        DBuf<double> de = h2d(c, eps, (size_t)n);
        std::unique_ptr<jues_cc> cc(new jues_cc());
        {
            Ctx::HostPhase ph(&c, "host:cc_create");
            cc->s = cc_create(&c, method, gp, n, co.p, o, cv.p, v, de.p, op);
        }
        Ctx::HostPhase ph(&c, "host:release_ao_eri");
        g.reset();
        *out = cc.release();
    });
}

int jues_cc_create_df(jues_ctx *ctx, const double *pqP, int pqP_is_device, int n, int naux, const double *Jpqh,
                      const double *Cocc, int o, const double *Cvir, int v, const double *eps,
                      const jues_cc_opts *opts, int variant, jues_cc **out) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        need(pqP, "pqP"); need(Cocc, "Cocc"); need(Cvir, "Cvir"); need(eps, "eps"); need(out, "out");
        *out = nullptr;
        check_dims(n, o, v);
        if (naux <= 0) throw Error(JUES_EINVAL, "naux must be positive");
        if (variant != JUES_DF_REFERENCE && variant != JUES_DF_RCCD) throw Error(JUES_EINVAL, "unknown DF variant");
        jues_cc_opts op;
        if (opts) op = *opts; else jues_cc_default_opts(&op);
        check_opts(op);
        cudaSetDevice(c.device);
        const int iprec = op.transform_precision >= 0 ? op.transform_precision : op.precision;
        DBuf<double> b = fitted_factor(c, pqP, pqP_is_device, n, naux, Jpqh, iprec);
        DBuf<double> co = h2d(c, Cocc, (size_t)n * o), cv = h2d(c, Cvir, (size_t)n * v);
        DBuf<double> de = h2d(c, eps, (size_t)n);
        std::unique_ptr<jues_cc> cc(new jues_cc());
        cc->s = cc_create_df(&c, b.p, n, naux, co.p, o, cv.p, v, de.p, op, variant == JUES_DF_REFERENCE);
        *out = cc.release();
    });
}

int jues_cc_iterate(jues_cc *cc, int nsweeps, int *done, int *converged) {
    return guarded([&] {
        need(cc, "cc");
        if (nsweeps < 0) throw Error(JUES_EINVAL, "nsweeps must be >= 0");
        cudaSetDevice(cc->s->ctx->device);
        cc_iterate(cc->s, nsweeps, done, converged);
    });
}

int jues_cc_set_precision(jues_cc *cc, int precision) {
    return guarded([&] {
        need(cc, "cc");
        if (!valid_precision(precision))
            throw Error(JUES_EINVAL, "unknown precision");
        cc->s->precision = precision;
        cc->s->refine_left = -1;
    });
}

int jues_cc_energy(jues_cc *cc, double *e_out) {
    return guarded([&] {
        need(cc, "cc"); need(e_out, "e_out");
        *e_out = cc->s->energy;
    });
}

int jues_cc_amplitudes(jues_cc *cc, double *t1_out, double *t2_out) {
    return guarded([&] {
        need(cc, "cc");
        cudaSetDevice(cc->s->ctx->device);
        cc_amplitudes(cc->s, t1_out, t2_out);
    });
}

int jues_cc_log(jues_cc *cc, jues_iter_log *log, int log_cap, int *count) {
    return guarded([&] {
        need(cc, "cc");
        int m = (int)cc->s->log.size();
        if (count) *count = m;
        if (log)
            for (int k = 0; k < m && k < log_cap; ++k) log[k] = cc->s->log[k];
    });
}

int jues_cc_destroy(jues_cc *cc) {
    return guarded([&] {
        need(cc, "cc");
        cudaSetDevice(cc->s->ctx->device);
        delete cc;
    });
}

// runs a created session to completion and fills the outputs
static int cc_run(jues_cc *cc, const jues_cc_opts *opts, double *e_out, double *t1_out, double *t2_out,
                  jues_iter_log *log, int log_cap, int *niter) {
    int st = 0;
    jues_cc_opts op;
    if (opts) op = *opts; else jues_cc_default_opts(&op);
    int done = 0, conv = 0;
    st = jues_cc_iterate(cc, op.maxit, &done, &conv);
    if (!st && e_out) st = jues_cc_energy(cc, e_out);
    if (!st && (t1_out || t2_out)) st = jues_cc_amplitudes(cc, t1_out, t2_out);
    if (!st && log) st = jues_cc_log(cc, log, log_cap, nullptr);
    if (niter) *niter = cc ? (int)cc->s->iters : 0;
    jues_cc_destroy(cc);
    if (!st && !conv && (op.r_conv > 0 || op.e_conv > 0) && op.maxit > 0) {
        set_last_error("CC iterations did not converge within maxit");
        st = JUES_ENOTCONV;
    }
    return st;
}

int jues_get_fock(jues_ctx *ctx, const double *gao, const double *hao, int n, const double *C, int nmo, int nocc,
                  double *f_out) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        need(gao, "gao"); need(hao, "hao"); need(C, "C"); need(f_out, "f_out");
        if (n <= 0 || nmo <= 0 || nmo > n || nocc < 0 || nocc > nmo)
            throw Error(JUES_EINVAL, "need 0 < nmo <= nbf and 0 <= nocc <= nmo");
        cudaSetDevice(c.device);
        const size_t nn = (size_t)n * n;
        DBuf<double> g = h2d(c, gao, nn * nn), h = h2d(c, hao, nn), cm = h2d(c, C, (size_t)n * nmo);
        DBuf<double> f(&c, (size_t)nmo * nmo);
        get_fock(&c, g.p, h.p, n, cm.p, nmo, cm.p, nocc, f.p);
        d2h(c, f_out, f.p, (size_t)nmo * nmo);
        c.check_flags();
    });
}

int jues_auto_rccsd(jues_ctx *ctx, const double *gao, const double *hao, int n, const double *C, int nmo, int ndocc,
                    int fcn, const jues_cc_opts *opts, int do_pT, double *e_out, double *ept_out, double *t1_out,
                    double *t2_out, jues_iter_log *log, int log_cap, int *niter) {
    jues_cc *cc = nullptr;
    int st = guarded([&] {
        Ctx &c = CX(ctx);
        need(gao, "gao"); need(hao, "hao"); need(C, "C");
        jues_cc_opts op;
        if (opts) op = *opts; else jues_cc_default_opts(&op);
        check_opts(op);
        cudaSetDevice(c.device);
        const size_t nn = (size_t)n * n;
        if (n <= 0 || nmo <= 0 || nmo > n) throw Error(JUES_EINVAL, "need 0 < nmo <= nbf");
        DBuf<double> g = h2d(c, gao, nn * nn), h = h2d(c, hao, nn), cm = h2d(c, C, (size_t)n * nmo);
        std::unique_ptr<jues_cc> p(new jues_cc());
        p->s = cc_create_auto(&c, g.p, h.p, n, cm.p, nmo, ndocc, fcn, op);
        cc = p.release();
    });
    if (st) return st;
    if (do_pT && ept_out) {
        // run the iterations, then (T) on the session before it is destroyed
        jues_cc_opts op;
        if (opts) op = *opts; else jues_cc_default_opts(&op);
        int done = 0, conv = 0;
        st = jues_cc_iterate(cc, op.maxit, &done, &conv);
        if (!st && e_out) st = jues_cc_energy(cc, e_out);
        if (!st && (t1_out || t2_out)) st = jues_cc_amplitudes(cc, t1_out, t2_out);
        if (!st && log) st = jues_cc_log(cc, log, log_cap, nullptr);
        if (!st) st = jues_cc_pT(cc, op.precision, ept_out);
        if (niter) *niter = (int)cc->s->iters;
        jues_cc_destroy(cc);
        if (!st && !conv && (op.r_conv > 0 || op.e_conv > 0) && op.maxit > 0) {
            set_last_error("CC iterations did not converge within maxit");
            st = JUES_ENOTCONV;
        }
        return st;
    }
    return cc_run(cc, opts, e_out, t1_out, t2_out, log, log_cap, niter);
}

int jues_pT(jues_ctx *ctx, const double *T1, const double *T2, const double *Vvvvo, const double *Vvooo,
            const double *Vvovo, const double *fo, const double *fv, int o, int v, int precision, double *e_out) {
    return guarded([&] {
        Ctx &c = CX(ctx);
        need(T1, "T1"); need(T2, "T2"); need(Vvvvo, "Vvvvo"); need(Vvooo, "Vvooo"); need(Vvovo, "Vvovo");
        need(fo, "fo"); need(fv, "fv"); need(e_out, "e_out");
        if (o <= 0 || v <= 0) throw Error(JUES_EINVAL, "need o > 0 and v > 0");
        if (!valid_precision(precision))
            throw Error(JUES_EINVAL, "unknown precision");
        cudaSetDevice(c.device);
        const size_t O = (size_t)o, V = (size_t)v;
        DBuf<double> t1 = h2d(c, T1, O * V), t2 = h2d(c, T2, O * O * V * V);
        DBuf<double> vv = h2d(c, Vvvvo, V * V * V * O), vo = h2d(c, Vvooo, V * O * O * O);
        DBuf<double> vvo = h2d(c, Vvovo, V * O * V * O);
        DBuf<double> dfo = h2d(c, fo, O), dfv = h2d(c, fv, V);
        *e_out = pT_energy(&c, precision, t1.p, t2.p, col_major(vv.p, v, v, v), col_major(vo.p, v, o, o),
                           col_major(vvo.p, v, o, v), dfo.p, dfv.p, o, v);
    });
}

int jues_cc_pT(jues_cc *cc, int precision, double *e_out) {
    return guarded([&] {
        need(cc, "cc"); need(e_out, "e_out");
        CCState *s = cc->s;
        if (s->method != 1) throw Error(JUES_EINVAL, "(T) needs a CCSD session");
        if (!valid_precision(precision))
            throw Error(JUES_EINVAL, "unknown precision");
        cudaSetDevice(s->ctx->device);
        const long long o = s->o, v = s->v, oo = o * o, ov = o * v;
        // AutoRCCSD.jl:295-297 as strided views of the physicists' blocks:
        // Vvvvo[a,b,c,i] = ovvv[i,b,c,a], Vvooo[a,j,i,k] = ooov[i,j,k,a], Vvovo[a,i,b,j] = oovv[i,j,a,b]
        View4 vv, vo, vvo;
        vv.p = s->ovvv.p; vv.s[0] = ov * v; vv.s[1] = o; vv.s[2] = ov; vv.s[3] = 1;
        vo.p = s->ooov.p; vo.s[0] = oo * o; vo.s[1] = o; vo.s[2] = 1; vo.s[3] = oo;
        vvo.p = s->oovv.p; vvo.s[0] = oo; vvo.s[1] = 1; vvo.s[2] = oo * v; vvo.s[3] = o;
        *e_out = pT_energy(s->ctx, precision, s->t1.p, s->T.p, vv, vo, vvo, s->eps.p, s->eps.p + o, (int)o, (int)v);
    });
}

static int cc_solve(jues_ctx *ctx, int method, const double *gao, int n, const double *Cocc, int o,
                    const double *Cvir, int v, const double *eps, const jues_cc_opts *opts, double *e_out,
                    double *t1_out, double *t2_out, jues_iter_log *log, int log_cap, int *niter) {
    jues_cc *cc = nullptr;
    int st = jues_cc_create(ctx, method, gao, 0, n, Cocc, o, Cvir, v, eps, opts, &cc);
    if (st) return st;
    return cc_run(cc, opts, e_out, t1_out, t2_out, log, log_cap, niter);
}

int jues_df_rccd(jues_ctx *ctx, const double *pqP, int n, int naux, const double *Jpqh, const double *Cocc, int o,
                 const double *Cvir, int v, const double *eps, const jues_cc_opts *opts, int variant, double *e_out,
                 double *t2_out, jues_iter_log *log, int log_cap, int *niter) {
    jues_cc *cc = nullptr;
    int st = jues_cc_create_df(ctx, pqP, 0, n, naux, Jpqh, Cocc, o, Cvir, v, eps, opts, variant, &cc);
    if (st) return st;
    return cc_run(cc, opts, e_out, nullptr, t2_out, log, log_cap, niter);
}

int jues_rccd(jues_ctx *ctx, const double *gao, int n, const double *Cocc, int o, const double *Cvir, int v,
              const double *eps, const jues_cc_opts *opts, double *e_out, double *t2_out, jues_iter_log *log,
              int log_cap, int *niter) {
    return cc_solve(ctx, 0, gao, n, Cocc, o, Cvir, v, eps, opts, e_out, nullptr, t2_out, log, log_cap, niter);
}

int jues_rccsd(jues_ctx *ctx, const double *gao, int n, const double *Cocc, int o, const double *Cvir, int v,
               const double *eps, const jues_cc_opts *opts, double *e_out, double *t1_out, double *t2_out,
               jues_iter_log *log, int log_cap, int *niter) {
    return cc_solve(ctx, 1, gao, n, Cocc, o, Cvir, v, eps, opts, e_out, t1_out, t2_out, log, log_cap, niter);
}

}  // extern "C"
