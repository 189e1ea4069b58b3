// Batched closed-shell MP2 energy and adjoint for many independent systems of uneven size.
//
// Every system's four-index transform, MP2 energy / Gamma seed, back-transform and dE/dC
// contractions are laid out in one device arena.  Step k of every system forms one grouped,
// persistent GETT launch (a tile list spanning all systems): 4 forward quarters, the
// energy/Gamma kernels, 4 back-transform quarters, 3 steps of the two three-quarter transforms
// and the final dE/dC contractions.  Each stage runs either as the grouped FP64 GETT with one of
// four tile shapes or, in split precision, as the grouped three-plane tcgen05 GEMM (two grouped
// operand packs and one persistent launch; stages whose contractions all have K <= 64).  The
// form of each stage is chosen by timing the candidates with CUDA events on first use
// (autotuning); the sequence is then captured once into a CUDA graph and replayed, and both the
// plan and the graph are cached by the batch signature (the list of (nbf, nocc), the requested
// outputs and the precision).
#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "common.cuh"
#include "staging.cuh"
#include "gett_f64.cuh"
#include "transform.cuh"

namespace jues {

namespace {

struct SysDesc {
    const double *K;     // (ia|jb) chemists' [i,a,j,b]
    const double *eps;
    double *G;           // Gamma
    double *e;           // energy slot
    int o, v;
    double e_bar;
    long long block0;    // first block of this system in mp2_gamma_grouped's grid
    int nblocks;         // its blocks
    int pairs_per_block; // (a <= b) pairs per block
};

// pair index p (a <= b) -> (a, b)
__device__ __forceinline__ void pair_of(long long p, int &a, int &b) {
    long long bb = (long long)((sqrt(8.0 * (double)p + 1.0) - 1.0) * 0.5);
    while (bb * (bb + 1) / 2 > p) --bb;
    while ((bb + 1) * (bb + 2) / 2 <= p) ++bb;
    b = (int)bb;
    a = (int)(p - bb * (bb + 1) / 2);
}

__device__ __forceinline__ double block_total(double acc) {
    __shared__ double red[32];
    for (int d = 16; d > 0; d >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, d);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int d = 16; d > 0; d >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, d);
    }
    return acc;
}

// Gamma = 2 e_bar (2K_iajb - K_ibja)/D and the energy's partial sums.  Each block takes a run of
// (a <= b) pairs of one system (several blocks per large system, so the largest systems do not
// serialise on one block); for a pair both K[:,a,:,b] and K[:,b,:,a] are read once.  The block's
// energy partial goes to part[block]; mp2_energy_grouped adds them per system in block order.
__global__ void __launch_bounds__(256) mp2_gamma_grouped(const SysDesc *__restrict__ sys, int nsys,
                                                         double *__restrict__ part) {
    const long long blk = blockIdx.x;
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sys[mid].block0 <= blk) lo = mid; else hi = mid - 1;
    }
    const SysDesc &S = sys[lo];
    const int o = S.o, v = S.v, oo = o * o;
    const long long ov = (long long)o * v;
    const long long npair = (long long)v * (v + 1) / 2;
    const long long p0 = (blk - S.block0) * S.pairs_per_block;
    const long long p1 = min(npair, p0 + S.pairs_per_block);
    const double two_ebar = 2.0 * S.e_bar;
    double acc = 0.0;
    for (long long t = threadIdx.x; t < (p1 - p0) * oo; t += blockDim.x) {
        const long long p = p0 + t / oo;
        const int ij = (int)(t % oo), i = ij % o, j = ij / o;
        int a, b;
        pair_of(p, a, b);
        const long long x_off = i + (long long)o * a + ov * j + ov * o * b;   // K[i,a,j,b]
        const long long y_off = i + (long long)o * b + ov * j + ov * o * a;   // K[i,b,j,a]
        const double inv = 1.0 / (S.eps[i] + S.eps[j] - S.eps[o + a] - S.eps[o + b]);
        const double x = S.K[x_off];
        if (a == b) {
            acc = fma(x * x, inv, acc);
            S.G[x_off] = two_ebar * x * inv;
        } else {
            const double y = S.K[y_off];
            acc = fma(x * (2.0 * x - y) + y * (2.0 * y - x), inv, acc);
            S.G[x_off] = two_ebar * (2.0 * x - y) * inv;
            S.G[y_off] = two_ebar * (2.0 * y - x) * inv;
        }
    }
    acc = block_total(acc);
    if (threadIdx.x == 0) part[blk] = acc;
}

// one block per system: its blocks' partial energies added in block order (deterministic)
__global__ void __launch_bounds__(256) mp2_energy_grouped(const SysDesc *__restrict__ sys,
                                                          const double *__restrict__ part) {
    const SysDesc &S = sys[blockIdx.x];
    double acc = 0.0;
    for (int k = threadIdx.x; k < S.nblocks; k += blockDim.x) acc += part[S.block0 + k];
    acc = block_total(acc);
    if (threadIdx.x == 0) *S.e = acc;
}

// tile shape index kShapeTC: the grouped three-plane tcgen05 GEMM (gett_tc.cu)
constexpr int kShapeTC = kNumTileShapes;

struct Stage {
    std::vector<GroupProblem> probs;
    std::vector<GettArgs> args;   // the same problems, for the grouped tcgen05 form
    DBuf<GroupProblem> dev;
    TcGroup *tc = nullptr;        // built when the batch runs split precision and every K <= 64
    long long total = 0;
    int shape = 0;
    std::string name;
    Stage() = default;
    Stage(Stage &&o) noexcept
        : probs(std::move(o.probs)), args(std::move(o.args)), dev(std::move(o.dev)), tc(o.tc), total(o.total),
          shape(o.shape), name(std::move(o.name)) {
        o.tc = nullptr;
    }
    Stage &operator=(Stage &&) = delete;
    ~Stage() { tc_group_destroy(tc); }
};

}  // namespace

struct BatchPlan {
    std::string key;
    DBuf<double> arena;
    std::vector<size_t> off_g, off_C, off_eps, off_gb, off_cb;
    std::vector<int> n, o;
    std::vector<Stage> stages;      // grouped GETT stages in order; energy runs after stage 4
    DBuf<SysDesc> sys;
    DBuf<double> energies, epart;
    long long gamma_blocks = 0;
    int n_forward = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    size_t graph_nodes = 0;
    ~BatchPlan() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

struct BatchCache {
    std::map<std::string, std::unique_ptr<BatchPlan>> plans;
};

void batch_cache_destroy(BatchCache *c) { delete c; }

static void run_stage(Ctx *ctx, Stage &st) {
    if (st.shape == kShapeTC)
        tc_group_run(ctx, st.tc);
    else
        gett_f64_grouped_launch(ctx, st.dev.p, (int)st.probs.size(), st.total, st.shape, st.name.c_str());
}

static void run_gamma(Ctx *ctx, BatchPlan &bp) {
    Ctx::Scope s(ctx, "batch_mp2_gamma");
    mp2_gamma_grouped<<<(unsigned)bp.gamma_blocks, 256, 0, ctx->stream>>>(bp.sys.p, (int)bp.n.size(), bp.epart.p);
    JUES_CHECK_CUDA(cudaGetLastError());
    mp2_energy_grouped<<<(unsigned)bp.n.size(), 256, 0, ctx->stream>>>(bp.sys.p, bp.epart.p);
    ctx->count_launch();
    JUES_CHECK_CUDA(cudaGetLastError());
}

static void run_stages(Ctx *ctx, BatchPlan &bp) {
    for (size_t k = 0; k < bp.stages.size(); ++k) {
        run_stage(ctx, bp.stages[k]);
        if ((int)k + 1 == bp.n_forward) run_gamma(ctx, bp);
    }
}

static void upload_stage(Ctx *ctx, Stage &st) {
    st.total = grouped_tiles(st.probs, st.shape);
    if (st.dev.n < st.probs.size()) st.dev = DBuf<GroupProblem>(ctx, st.probs.size());
    JUES_CHECK_CUDA(cudaMemcpyAsync(st.dev.p, st.probs.data(), st.probs.size() * sizeof(GroupProblem),
                                    cudaMemcpyHostToDevice, ctx->stream));
}

// time each tile shape on the real stage (inputs already in the arena) and keep the fastest
static void autotune(Ctx *ctx, BatchPlan &bp) {
    cudaEvent_t e0, e1;
    JUES_CHECK_CUDA(cudaEventCreate(&e0));
    JUES_CHECK_CUDA(cudaEventCreate(&e1));
    for (size_t k = 0; k < bp.stages.size(); ++k) {
        Stage &st = bp.stages[k];
        float best = -1.f;
        int best_shape = 0;
        // the FP64 tile shapes, and the grouped tcgen05 form where it was built
        const int first = (ctx->batch_form == 2 && st.tc) ? kShapeTC : 0;
        const int last = (st.tc && ctx->batch_form != 1) ? kShapeTC : kNumTileShapes - 1;
        for (int sh = first; sh <= last; ++sh) {
            st.shape = sh;
            if (sh != kShapeTC) upload_stage(ctx, st);
            // warm once, then time
            run_stage(ctx, st);
            JUES_CHECK_CUDA(cudaEventRecord(e0, ctx->stream));
            run_stage(ctx, st);
            JUES_CHECK_CUDA(cudaEventRecord(e1, ctx->stream));
            JUES_CHECK_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            JUES_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (best < 0 || ms < best) { best = ms; best_shape = sh; }
        }
        st.shape = best_shape;
        if (st.shape != kShapeTC) upload_stage(ctx, st);
        // stages read what earlier stages wrote: run this one for real before tuning the next
        run_stage(ctx, st);
        if ((int)k + 1 == bp.n_forward) run_gamma(ctx, bp);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
}

static std::unique_ptr<BatchPlan> make_plan(Ctx *ctx, const std::string &key, int nsys, const jues_mp2_system *sys,
                                            double e_bar, bool want_gb, bool want_cb, bool split) {
    std::unique_ptr<BatchPlan> bp(new BatchPlan());
    bp->key = key;
    struct Off {
        size_t g, C, eps, K, G, b0, b1, b2, b3, H, Hp, gb, cb;
    };
    std::vector<Off> off(nsys);
    size_t top = 0;
    auto take = [&](long long cnt) {
        size_t at = top;
        top += ((size_t)cnt + 31) / 32 * 32;   // 256-byte alignment
        return at;
    };
    for (int s = 0; s < nsys; ++s) {
        const long long n = sys[s].n, o = sys[s].o, v = n - o;
        JUES_REQUIRE(n > 0 && o > 0 && v > 0, "batch system needs 0 < nocc < nbf");
        const long long n4 = n * n * n * n, ovov = o * v * o * v;
        const long long scratch = n * n * n * std::max(o, v);   // >= every intermediate below
        Off &f = off[s];
        f.g = take(n4);
        f.C = take(n * n);
        f.eps = take(n);
        f.K = take(ovov);
        f.G = take(ovov);
        f.b0 = take(scratch);
        f.b1 = take(scratch);
        f.b2 = want_cb ? take(scratch) : 0;
        f.b3 = want_cb ? take(scratch) : 0;
        f.H = want_cb ? take(n * v * o * v) : 0;
        f.Hp = want_cb ? take(o * n * o * v) : 0;
        f.gb = want_gb ? take(n4) : 0;
        f.cb = want_cb ? take(n * n) : 0;
        bp->n.push_back((int)n);
        bp->o.push_back((int)o);
        bp->off_g.push_back(f.g);
        bp->off_C.push_back(f.C);
        bp->off_eps.push_back(f.eps);
        bp->off_gb.push_back(f.gb);
        bp->off_cb.push_back(f.cb);
    }
    bp->arena = DBuf<double>(ctx, top);
    double *A = bp->arena.p;
    std::vector<Stage> fwd(4), bwd(4), third(3), fin(1);
    std::vector<SysDesc> descs(nsys);
    bp->energies = DBuf<double>(ctx, nsys);
    for (int s = 0; s < nsys; ++s) {
        const Off &f = off[s];
        const int n = bp->n[s], o = bp->o[s], v = n - o;
        const long long ov = (long long)o * v;
        const double *Co = A + f.C, *Cv = A + f.C + (size_t)n * o;
        {
            const double *Cs[4] = {Co, Cv, Co, Cv};
            int d[4] = {o, v, o, v};
            long long ostr[4] = {1, o, ov, ov * o};
            auto st = transform4_plan(A + f.g, n, Cs, d, A + f.K, ostr, A + f.b0, A + f.b1);
            for (int k = 0; k < 4; ++k) {
                fwd[k].probs.push_back(to_problem(st[k]));
                fwd[k].args.push_back(st[k]);
            }
        }
        {
            const long long npair = (long long)v * (v + 1) / 2;
            const int ppb = std::max(1, 2048 / (o * o));
            const int nb = (int)((npair + ppb - 1) / ppb);
            descs[s] = SysDesc{A + f.K, A + f.eps, A + f.G, bp->energies.p + s, o, v, e_bar, bp->gamma_blocks, nb, ppb};
            bp->gamma_blocks += nb;
        }
        if (want_gb) {
            const double *Cs[4] = {Co, Cv, Co, Cv};
            int d[4] = {o, v, o, v};
            auto st = backtransform4_plan(A + f.G, d, n, Cs, A + f.gb, A + f.b0, A + f.b1);
            for (int k = 0; k < 4; ++k) {
                bwd[k].probs.push_back(to_problem(st[k]));
                bwd[k].args.push_back(st[k]);
            }
        }
        if (want_cb) {
            // H = (mu a|j b) with scratch b0/b1 and H' = (i nu|j b) with scratch b2/b3: step k of
            // both runs in the same grouped launch; the back-transform (if any) is done with
            // b0/b1 by then
            const double *C1[4] = {nullptr, Cv, Co, Cv};
            int d1[4] = {n, v, o, v};
            long long os1[4] = {1, n, (long long)n * v, (long long)n * v * o};
            auto h = transform4_plan(A + f.g, n, C1, d1, A + f.H, os1, A + f.b0, A + f.b1);
            const double *C2[4] = {Co, nullptr, Co, Cv};
            int d2[4] = {o, n, o, v};
            long long os2[4] = {1, o, (long long)o * n, (long long)o * n * o};
            auto hp = transform4_plan(A + f.g, n, C2, d2, A + f.Hp, os2, A + f.b2, A + f.b3);
            for (int k = 0; k < 3; ++k) {
                third[k].probs.push_back(to_problem(h[k]));
                third[k].probs.push_back(to_problem(hp[k]));
                third[k].args.push_back(h[k]);
                third[k].args.push_back(hp[k]);
            }
            GettArgs a;   // dE/dC[mu,i] = 2 sum_{ajb} H[mu,(ajb)] G[i,(ajb)]
            a.M = n; a.N = o; a.K = ov * v;
            a.alpha = 2.0; a.beta = 0.0;
            a.A = A + f.H; a.mA = plain(1); a.kA = plain(n);
            a.B = A + f.G; a.kB = plain(o); a.nB = plain(1);
            a.C = A + f.cb; a.mC = plain(1); a.nC = plain(n);
            a.Cin = nullptr;
            fin[0].probs.push_back(to_problem(a));
            fin[0].args.push_back(a);
            GettArgs b;   // dE/dC[nu,a] = 2 sum_{ijb} H'[i,nu,j,b] G[i,a,j,b]
            b.M = n; b.N = v; b.K = (long long)o * o * v;
            b.alpha = 2.0; b.beta = 0.0;
            b.A = A + f.Hp; b.mA = plain(o); b.kA = mode3(o, o, 1, (long long)o * n, (long long)o * n * o);
            b.B = A + f.G; b.kB = mode3(o, o, 1, ov, ov * o); b.nB = plain(o);
            b.C = A + f.cb + (size_t)n * o; b.mC = plain(1); b.nC = plain(n);
            b.Cin = nullptr;
            fin[0].probs.push_back(to_problem(b));
            fin[0].args.push_back(b);
        }
    }
    for (auto &st : fwd) { st.name = "batch_transform"; bp->stages.push_back(std::move(st)); }
    bp->n_forward = 4;
    if (want_gb)
        for (auto &st : bwd) { st.name = "batch_backtransform"; bp->stages.push_back(std::move(st)); }
    if (want_cb) {
        for (auto &st : third) { st.name = "batch_third_quarter"; bp->stages.push_back(std::move(st)); }
        fin[0].name = "batch_cbar";
        bp->stages.push_back(std::move(fin[0]));
    }
    bp->sys = DBuf<SysDesc>(ctx, nsys);
    bp->epart = DBuf<double>(ctx, (size_t)bp->gamma_blocks);
    JUES_CHECK_CUDA(cudaMemcpyAsync(bp->sys.p, descs.data(), nsys * sizeof(SysDesc), cudaMemcpyHostToDevice,
                                    ctx->stream));
    // split precision: every stage whose contractions all have K <= 64 (every stage but the final
    // dE/dC one when nbf <= 64) gets the grouped three-plane tcgen05 form as a tuning candidate
    if (split)
        for (Stage &st : bp->stages) st.tc = tc_group_build(ctx, st.args, (st.name + "_tc").c_str());
    return bp;
}

static std::string signature(int nsys, const jues_mp2_system *sys, double e_bar, bool gb, bool cb, bool split,
                             int form) {
    std::string k = std::to_string(nsys) + (gb ? "G" : "g") + (cb ? "C" : "c") + (split ? "S" : "D") +
                    std::to_string(form) + "," + std::to_string(e_bar);
    for (int s = 0; s < nsys; ++s) k += "," + std::to_string(sys[s].n) + ":" + std::to_string(sys[s].o);
    return k;
}

void batch_rmp2(Ctx *ctx, int nsys, const jues_mp2_system *sys, int precision, double e_bar, double *e_out,
                double **gao_bar, double **C_bar, jues_batch_info *info) {
    JUES_REQUIRE(nsys > 0, "nsys must be positive");
    JUES_REQUIRE(valid_precision(precision), "unknown precision");
    const bool split = is_split(precision);
    for (int s = 0; s < nsys; ++s) {
        JUES_REQUIRE(sys[s].gao && sys[s].C && sys[s].eps, "null pointer in a batch system");
        JUES_REQUIRE(sys[s].n > 0 && sys[s].o > 0 && sys[s].o < sys[s].n, "batch system needs 0 < nocc < nbf");
    }
    bool want_gb = false, want_cb = false;
    for (int s = 0; s < nsys; ++s) {
        want_gb = want_gb || (gao_bar && gao_bar[s]);
        want_cb = want_cb || (C_bar && C_bar[s]);
    }
    if (!ctx->batch) ctx->batch = new BatchCache();
    const std::string key = signature(nsys, sys, e_bar, want_gb, want_cb, split, ctx->batch_form);
    auto it = ctx->batch->plans.find(key);
    bool fresh = false;
    if (it == ctx->batch->plans.end()) {
        ctx->batch->plans.clear();   // one resident plan per context keeps memory bounded
        it = ctx->batch->plans.emplace(key, make_plan(ctx, key, nsys, sys, e_bar, want_gb, want_cb, split)).first;
        fresh = true;
    }
    BatchPlan &bp = *it->second;
    cudaEvent_t t0, t1, t2, t3;
    JUES_CHECK_CUDA(cudaEventCreate(&t0));
    JUES_CHECK_CUDA(cudaEventCreate(&t1));
    JUES_CHECK_CUDA(cudaEventCreate(&t2));
    JUES_CHECK_CUDA(cudaEventCreate(&t3));
    JUES_CHECK_CUDA(cudaEventRecord(t0, ctx->stream));
    double *A = bp.arena.p;
    // the systems' inputs through the staging ring (no page-locking of the caller's arrays)
    std::vector<HostSeg> ups;
    ups.reserve(3 * (size_t)nsys);
    for (int s = 0; s < nsys; ++s) {
        const size_t n = (size_t)sys[s].n;
        ups.push_back({A + bp.off_g[s], sys[s].gao, n * n * n * n * sizeof(double)});
        ups.push_back({A + bp.off_C[s], sys[s].C, n * n * sizeof(double)});
        ups.push_back({A + bp.off_eps[s], sys[s].eps, n * sizeof(double)});
    }
    staged_h2d(ctx, ups);
    JUES_CHECK_CUDA(cudaEventRecord(t1, ctx->stream));
    if (fresh) {
        autotune(ctx, bp);   // runs every stage once on the uploaded data
        const bool prof = ctx->profiling;
        ctx->profiling = false;   // no event records inside the capture
        JUES_CHECK_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        try {
            run_stages(ctx, bp);
        } catch (...) {
            cudaGraph_t g;
            cudaStreamEndCapture(ctx->stream, &g);
            if (g) cudaGraphDestroy(g);
            ctx->profiling = prof;
            throw;
        }
        JUES_CHECK_CUDA(cudaStreamEndCapture(ctx->stream, &bp.graph));
        ctx->profiling = prof;
        JUES_CHECK_CUDA(cudaGraphInstantiate(&bp.exec, bp.graph, 0));
        JUES_CHECK_CUDA(cudaGraphGetNodes(bp.graph, nullptr, &bp.graph_nodes));
    }
    JUES_CHECK_CUDA(cudaEventRecord(t1, ctx->stream));
    JUES_CHECK_CUDA(cudaGraphLaunch(bp.exec, ctx->stream));
    ctx->launches += (long long)bp.graph_nodes;
    JUES_CHECK_CUDA(cudaEventRecord(t2, ctx->stream));
    JUES_CHECK_CUDA(cudaMemcpyAsync(e_out, bp.energies.p, nsys * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    std::vector<HostSeg> down;
    for (int s = 0; s < nsys; ++s) {
        const size_t n = (size_t)sys[s].n;
        if (want_gb && gao_bar[s]) down.push_back({gao_bar[s], A + bp.off_gb[s], n * n * n * n * sizeof(double)});
        if (want_cb && C_bar[s]) down.push_back({C_bar[s], A + bp.off_cb[s], n * n * sizeof(double)});
    }
    staged_d2h(ctx, down);   // returns with the data in the caller's arrays
    JUES_CHECK_CUDA(cudaEventRecord(t3, ctx->stream));
    JUES_CHECK_CUDA(cudaEventSynchronize(t3));
    float up = 0.f, gr = 0.f, dn = 0.f;
    cudaEventElapsedTime(&up, t0, t1);
    cudaEventElapsedTime(&gr, t1, t2);
    cudaEventElapsedTime(&dn, t2, t3);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaEventDestroy(t2);
    cudaEventDestroy(t3);
    if (info) {
        info->upload_ms = up;
        info->graph_ms = gr;
        info->download_ms = dn;
        info->graph_nodes = (int)bp.graph_nodes;
        info->tuned = fresh ? 1 : 0;
        info->nstages = (int)bp.stages.size();
        for (int k = 0; k < 16; ++k) info->tile_shape[k] = k < (int)bp.stages.size() ? bp.stages[k].shape : -1;
    }
    ctx->check_flags();
}

}  // namespace jues
