// AO->MO four-index transformation (Transformation.jl:39-93, IntegralTransformation.jl:38-101).
//
// out[i,a,j,b] = sum C1[mu,i] C2[nu,a] C3[lam,j] C4[sig,b] g[mu,nu,lam,sig] is evaluated as four
// quarter transforms, each one GEMM over composite tensor modes (no explicit permutes).  The
// reference always contracts sigma first (C4); the result does not depend on the order, so the
// quarter with the smallest MO dimension goes first, which minimises the flops
// (F = sum_k 2 n^(5-k) prod_{m<=k} d_(m)).  The last quarter writes straight into the caller's
// layout: chemists' [i,a,j,b] or, for get_eri's physicists' notation, [i,j,a,b].
#include <algorithm>
#include <string>
#include <utility>
#include <vector>

#include "common.cuh"
#include "transform.cuh"

namespace jues {

double transform4_flops(int n, const int d[4]) {
    int s[4] = {d[0], d[1], d[2], d[3]};
    std::sort(s, s + 4);
    double f = 0.0, prod = 1.0, np = (double)n * n * n * n;
    for (int k = 0; k < 4; ++k) {
        prod *= s[k];
        np /= n;
        f += 2.0 * np * n * prod;   // 2 n^(5-k) prod d
    }
    return f;
}

std::vector<GettArgs> transform4_plan(const double *g, int n, const double *const C[4], const int d_in[4],
                                      double *out, const long long ostr[4], double *buf0, double *buf1,
                                      const long long *din) {
    // a null C[p] keeps index p as it is in the input: an AO index (three-quarter transforms for
    // the MP2 adjoint) or, with input extents din, an index an earlier step already transformed
    long long dims[4] = {n, n, n, n};
    if (din)
        for (int p = 0; p < 4; ++p) dims[p] = din[p];
    int d[4];
    for (int p = 0; p < 4; ++p) {
        d[p] = C[p] ? d_in[p] : (int)dims[p];
        JUES_REQUIRE(d[p] >= 0, "negative MO dimension");
        JUES_REQUIRE(!C[p] || dims[p] == n, "only AO indices are transformed");
    }
    std::vector<GettArgs> steps;
    if (d[0] == 0 || d[1] == 0 || d[2] == 0 || d[3] == 0) return steps;
    int nsteps = 0;
    for (int p = 0; p < 4; ++p) nsteps += C[p] ? 1 : 0;
    JUES_REQUIRE(nsteps > 0, "transform4 needs at least one coefficient matrix");
    bool done[4];
    for (int p = 0; p < 4; ++p) done[p] = !C[p];
    const double *cur = g;
    double *bufs[2] = {buf0, buf1};
    int which = 0;
    for (int step = 0; step < nsteps; ++step) {
        int p = -1;
        for (int q = 0; q < 4; ++q)
            if (!done[q] && (p < 0 || d[q] < d[p])) p = q;
        long long sX[4], nd[4], sY[4];
        sX[0] = 1;
        for (int q = 1; q < 4; ++q) sX[q] = sX[q - 1] * dims[q - 1];
        for (int q = 0; q < 4; ++q) nd[q] = dims[q];
        nd[p] = d[p];
        double *dst;
        if (step == nsteps - 1) {
            for (int q = 0; q < 4; ++q) sY[q] = ostr[q];
            dst = out;
        } else {
            sY[0] = 1;
            for (int q = 1; q < 4; ++q) sY[q] = sY[q - 1] * nd[q - 1];
            dst = bufs[which];
        }
        int q1 = -1, q2 = -1, q3 = -1;
        for (int q = 0; q < 4; ++q) {
            if (q == p) continue;
            if (q1 < 0) q1 = q; else if (q2 < 0) q2 = q; else q3 = q;
        }
        GettArgs a;
        a.M = dims[q1] * dims[q2] * dims[q3];
        a.N = d[p];
        a.K = n;
        a.alpha = 1.0;
        a.beta = 0.0;
        a.A = cur;
        a.mA = mode3(dims[q1], dims[q2], sX[q1], sX[q2], sX[q3]);
        a.kA = plain(sX[p]);
        a.B = C[p];
        a.kB = plain(1);
        a.nB = plain(n);
        a.C = dst;
        a.mC = mode3(nd[q1], nd[q2], sY[q1], sY[q2], sY[q3]);
        a.nC = plain(sY[p]);
        steps.push_back(a);
        for (int q = 0; q < 4; ++q) dims[q] = nd[q];
        done[p] = true;
        cur = dst;
        which ^= 1;
    }
    return steps;
}

long long transform4_scratch(int n, const double *const C[4], const int d_in[4], const long long *din) {
    // largest intermediate of transform4_plan
    long long dims[4] = {n, n, n, n}, best = 0;
    if (din)
        for (int p = 0; p < 4; ++p) dims[p] = din[p];
    int d[4];
    for (int p = 0; p < 4; ++p) d[p] = C[p] ? d_in[p] : (int)dims[p];
    bool done[4];
    int nsteps = 0;
    for (int p = 0; p < 4; ++p) { done[p] = !C[p]; nsteps += C[p] ? 1 : 0; }
    for (int step = 0; step + 1 < nsteps; ++step) {
        int p = -1;
        for (int q = 0; q < 4; ++q)
            if (!done[q] && (p < 0 || d[q] < d[p])) p = q;
        dims[p] = d[p];
        done[p] = true;
        best = std::max(best, dims[0] * dims[1] * dims[2] * dims[3]);
    }
    return best;
}

void transform4(Ctx *ctx, int prec, const double *g, int n, const double *const C[4], const int d_in[4],
                double *out, const long long ostr[4], bool g_const, const long long *din) {
    const long long need = transform4_scratch(n, C, d_in, din);
    DBuf<double> b0(ctx, (size_t)need), b1(ctx, (size_t)need);
    std::vector<GettArgs> steps = transform4_plan(g, n, C, d_in, out, ostr, b0.p, b1.p, din);
    for (size_t k = 0; k < steps.size(); ++k) {
        steps[k].a_const = (k == 0) && g_const;
        gett(ctx, integral_precision(prec), steps[k], k == 0 ? "transform_q1" : "transform_q234");
    }
}

std::vector<GettArgs> backtransform4_plan(const double *X, const int d[4], int n, const double *const C[4],
                                          double *out, double *buf0, double *buf1) {
    // out[mu,nu,lam,sig] = sum X[i,a,j,b] C1[mu,i] C2[nu,a] C3[lam,j] C4[sig,b]; the last step
    // costs 2 n^4 d_last, so the largest MO dimension is expanded first
    long long dims[4] = {d[0], d[1], d[2], d[3]};
    bool done[4] = {false, false, false, false};
    const double *cur = X;
    double *bufs[2] = {buf0, buf1};
    int which = 0;
    std::vector<GettArgs> steps;
    for (int step = 0; step < 4; ++step) {
        int p = -1;
        for (int q = 0; q < 4; ++q)
            if (!done[q] && (p < 0 || d[q] > d[p])) p = q;
        long long sX[4], nd[4], sY[4];
        sX[0] = 1;
        for (int q = 1; q < 4; ++q) sX[q] = sX[q - 1] * dims[q - 1];
        for (int q = 0; q < 4; ++q) nd[q] = dims[q];
        nd[p] = n;
        sY[0] = 1;
        for (int q = 1; q < 4; ++q) sY[q] = sY[q - 1] * nd[q - 1];
        double *dst = step == 3 ? out : bufs[which];
        int q1 = -1, q2 = -1, q3 = -1;
        for (int q = 0; q < 4; ++q) {
            if (q == p) continue;
            if (q1 < 0) q1 = q; else if (q2 < 0) q2 = q; else q3 = q;
        }
        GettArgs a;
        a.M = dims[q1] * dims[q2] * dims[q3];
        a.N = n;
        a.K = d[p];
        a.alpha = 1.0;
        a.beta = 0.0;
        a.A = cur;
        a.mA = mode3(dims[q1], dims[q2], sX[q1], sX[q2], sX[q3]);
        a.kA = plain(sX[p]);
        a.B = C[p];            // B[k=d, n=mu] = C[mu, d]
        a.kB = plain(n);
        a.nB = plain(1);
        a.C = dst;
        a.mC = mode3(nd[q1], nd[q2], sY[q1], sY[q2], sY[q3]);
        a.nC = plain(sY[p]);
        steps.push_back(a);
        for (int q = 0; q < 4; ++q) dims[q] = nd[q];
        done[p] = true;
        cur = dst;
        which ^= 1;
    }
    return steps;
}

long long backtransform4_scratch(const int d[4], int n) {
    long long dims[4] = {d[0], d[1], d[2], d[3]}, best = 0;
    bool done[4] = {false, false, false, false};
    for (int step = 0; step < 3; ++step) {
        int p = -1;
        for (int q = 0; q < 4; ++q)
            if (!done[q] && (p < 0 || d[q] > d[p])) p = q;
        dims[p] = n;
        done[p] = true;
        best = std::max(best, dims[0] * dims[1] * dims[2] * dims[3]);
    }
    return best;
}

void backtransform4(Ctx *ctx, int prec, const double *X, const int d[4], int n, const double *const C[4],
                    double *out) {
    const long long need = backtransform4_scratch(d, n);
    DBuf<double> b0(ctx, (size_t)need), b1(ctx, (size_t)need);
    for (auto &a : backtransform4_plan(X, d, n, C, out, b0.p, b1.p))
        gett(ctx, integral_precision(prec), a, "backtransform");
}

namespace {
// coefficient matrices, MO extents and output strides of one get_eri block
struct EriReq {
    const double *C[4];
    int d[4];
    long long ostr[4];
    double *out;
};

EriReq eri_request(int n, const double *Cocc, int o, const double *Cvir, int v, const char spec_in[4], bool phys,
                   int fcn, double *out) {
    char s[4] = {spec_in[0], spec_in[1], spec_in[2], spec_in[3]};
    if (phys) { char t = s[1]; s[1] = s[2]; s[2] = t; }   // IntegralTransformation.jl:46-48
    EriReq r;
    r.out = out;
    for (int q = 0; q < 4; ++q) {
        char ch = s[q];
        if (ch == 'o' || ch == 'O') {
            JUES_REQUIRE(fcn >= 0 && fcn <= o, "fcn out of range");
            r.C[q] = Cocc + (size_t)fcn * n;   // drop the first fcn occupied columns (:54,58)
            r.d[q] = o - fcn;
        } else if (ch == 'v' || ch == 'V') {
            r.C[q] = Cvir;
            r.d[q] = v;
        } else {
            throw Error(JUES_EINVAL, std::string("Invalid string given to get_eri: ") + std::string(spec_in, 4));
        }
    }
    if (phys) {
        // chem positions (1,2,3,4) = (i,a,j,b) land in phys [i,j,a,b] with dims (d1,d3,d2,d4)
        r.ostr[0] = 1;
        r.ostr[2] = r.d[0];
        r.ostr[1] = (long long)r.d[0] * r.d[2];
        r.ostr[3] = (long long)r.d[0] * r.d[2] * r.d[1];
    } else {
        r.ostr[0] = 1;
        r.ostr[1] = r.d[0];
        r.ostr[2] = (long long)r.d[0] * r.d[1];
        r.ostr[3] = (long long)r.d[0] * r.d[1] * r.d[2];
    }
    return r;
}

// the index transform4_plan contracts next: the smallest MO extent among the indices still in
// the AO basis (the lowest position on a tie)
int next_index(const EriReq &r, const bool done[4]) {
    int p = -1;
    for (int q = 0; q < 4; ++q)
        if (!done[q] && (p < 0 || r.d[q] < r.d[p])) p = q;
    return p;
}

// Transform the requests that share the steps taken so far (X: their common intermediate with
// extents dims, done: the indices already transformed).  Requests whose next step coincides
// (same index, same coefficient matrix) take it once, into a new intermediate; a request alone
// in its group runs its remaining steps straight into its output.
void eri_tree(Ctx *ctx, int prec, const double *X, int n, const long long dims[4], const bool done[4],
              const std::vector<const EriReq *> &reqs, bool x_const, int nleft) {
    std::vector<bool> used(reqs.size(), false);
    for (size_t a = 0; a < reqs.size(); ++a) {
        if (used[a]) continue;
        const int p = next_index(*reqs[a], done);
        std::vector<const EriReq *> group;
        for (size_t b = a; b < reqs.size(); ++b)
            if (!used[b] && next_index(*reqs[b], done) == p && reqs[b]->C[p] == reqs[a]->C[p]) {
                group.push_back(reqs[b]);
                used[b] = true;
            }
        if (group.size() == 1 || nleft == 1) {
            for (const EriReq *r : group) {
                const double *C[4];
                for (int q = 0; q < 4; ++q) C[q] = done[q] ? nullptr : r->C[q];
                transform4(ctx, prec, X, n, C, r->d, r->out, r->ostr, x_const, dims);
            }
            continue;
        }
        // the shared step: index p of X contracted with C[p], natural strides
        long long nd[4] = {dims[0], dims[1], dims[2], dims[3]};
        nd[p] = group[0]->d[p];
        DBuf<double> H(ctx, (size_t)(nd[0] * nd[1] * nd[2] * nd[3]));
        {
            const double *C[4] = {nullptr, nullptr, nullptr, nullptr};
            C[p] = group[0]->C[p];
            const long long os[4] = {1, nd[0], nd[0] * nd[1], nd[0] * nd[1] * nd[2]};
            transform4(ctx, prec, X, n, C, group[0]->d, H.p, os, x_const, dims);
        }
        bool done2[4] = {done[0], done[1], done[2], done[3]};
        done2[p] = true;
        eri_tree(ctx, prec, H.p, n, nd, done2, group, true, nleft - 1);
    }
}
}  // namespace

void get_eri_block(Ctx *ctx, int prec, const double *g, int n, const double *Cocc, int o,
                   const double *Cvir, int v, const char spec_in[4], bool phys, int fcn, double *out,
                   bool g_const) {
    const EriReq r = eri_request(n, Cocc, o, Cvir, v, spec_in, phys, fcn, out);
    transform4(ctx, prec, g, n, r.C, r.d, out, r.ostr, g_const);
}

void get_eri_blocks(Ctx *ctx, int prec, const double *g, int n, const double *Cocc, int o, const double *Cvir,
                    int v, const std::vector<std::pair<std::string, double *>> &blocks, bool phys, int fcn,
                    bool g_const) {
    std::vector<EriReq> rs;
    for (const auto &b : blocks) {
        JUES_REQUIRE(b.first.size() == 4, "get_eri spec must have 4 characters");
        rs.push_back(eri_request(n, Cocc, o, Cvir, v, b.first.c_str(), phys, fcn, b.second));
    }
    std::vector<const EriReq *> ptrs;
    for (const EriReq &r : rs) ptrs.push_back(&r);
    const long long dims[4] = {n, n, n, n};
    const bool done[4] = {false, false, false, false};
    eri_tree(ctx, prec, g, n, dims, done, ptrs, g_const, 4);
}

}  // namespace jues
