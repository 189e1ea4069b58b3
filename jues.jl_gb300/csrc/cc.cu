// Closed-shell CCD / CCSD on the device: integrals, sweeps, DIIS, convergence.
//
// The equations are those of src/CoupledCluster/RCCD.jl:234-303 (== mRCCD.jl:301-394) and
// RCCSD.jl:187-289; intermediates as in RCCD.jl:169-467.  Every contraction is one GETT over
// composite tensor modes, so no permuted copies of T2 are made.  Three exact rewrites reduce the
// work without changing the result beyond rounding:
//   * Wabef is never formed: sum_ef T[ij,ef] Wabef[ab,ef] = T.vvvv^T + 1/2 X^T.T with
//     X[mn,ij] = sum_ef oovv[mn,ef] T[ij,ef]; X also gives Wmnij (= oooo + X/2), so the two
//     ladders become T.vvvv^T + (oooo + X)^T.T  (2o^2v^4 + 4o^4v^2 instead of 4o^2v^4 + 2o^4v^2);
//   * the terms of RCCD.jl:243-254 that are images of each other under (i,a)<->(j,b) are
//     computed once into Z and added as Z[i,j,a,b] + Z[j,i,b,a] by the finalisation kernel;
//   * the two Fmi terms, - T[i,m,a,b] Fmi[m,j] - T[m,j,a,b] Fmi[m,i], are hole-hole ladder
//     terms with W'[(m,n),(i,j)] -= [m = i] Fmi[n,j] + [n = j] Fmi[m,i], so they cost no GEMM
//     of their own (that one had K = o and needed its own operand pack of T2).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "cc.cuh"
#include "df.cuh"
#include "fock.cuh"
#include "transform.cuh"

namespace jues {

double ccd_sweep_flops(int o_, int v_) {
    double o = o_, v = v_;
    return 2 * o * o * v * v * v * v + 12 * o * o * o * v * v * v + 4 * o * o * o * o * v * v +
           4 * o * o * v * v * v + 2 * o * o * o * v * v;
}

double ccd_reference_flops(int o_, int v_) {
    double o = o_, v = v_;
    return 4 * o * o * v * v * v * v + 16 * o * o * o * v * v * v + 4 * o * o * o * o * v * v +
           6 * o * o * v * v * v + 6 * o * o * o * v * v;
}

namespace {

// C = alpha * A.B + beta * Cin over the given modes.  With s->cache_operands set, split-precision
// packs of every operand are kept until the operand's buffer is dropped (see ccd_sweep).
void G(CCState *s, int prec, const char *name, long long M, long long N, long long K, double alpha,
       const double *A, Mode mA, Mode kA, const double *B, Mode kB, Mode nB, double beta, double *C,
       Mode mC, Mode nC, const double *Cin = nullptr, bool a_const = false, bool b_const = false) {
    a_const = a_const || s->cache_operands;
    b_const = b_const || s->cache_operands;
    GettArgs g;
    g.M = M; g.N = N; g.K = K;
    g.alpha = alpha; g.beta = beta;
    g.A = A; g.mA = mA; g.kA = kA;
    g.B = B; g.kB = kB; g.nB = nB;
    g.C = C; g.mC = mC; g.nC = nC;
    g.Cin = Cin;
    g.a_const = a_const; g.b_const = b_const;
    gett(s->ctx, prec, g, name);
}

void d2d(Ctx *ctx, double *dst, const double *src, size_t n) {
    JUES_CHECK_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
}

// a non-owning view of n doubles of another buffer (no context: never freed through it)
DBuf<double> view_of(double *p, size_t n) {
    DBuf<double> d;
    d.p = p;
    d.n = n;
    return d;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// The ladders in split precision on K-stacked packs.  With ko = roundup(o^2, 128) and
// kv = roundup(v^2, 128):  X = oovv . Tl^T (Tl = T2, or T2 + tau for CCSD) reads Tl from the
// second block of stackLA; after W' is complete, one GEMM of K = ko + kv gives
// L = oovv + W'^T . Tl + Tl . vvvv^T (the hole-hole and particle-particle ladders).
// ---------------------------------------------------------------------------------------
static void ladder_stacks_x(CCState *s, const double *Tl, const char *name) {
    Ctx *ctx = s->ctx;
    const long long o = s->o, v = s->v, oo = o * o, vv = v * v;
    const long long ko = (oo + 127) / 128 * 128, kv = (vv + 127) / 128 * 128;
    if (!s->stackLB.buf.p) {
        s->stackLB.ensure(ctx, vv, ko + kv, 2);
        pack_stacked(ctx, s->stackLB, ko, s->vvvv.p, plain(1), plain(vv), vv, vv, 1.0);   // vvvv[ab, ef]
        s->stackXW.ensure(ctx, oo, kv, 2);
        pack_stacked(ctx, s->stackXW, 0, s->oovv.p, plain(1), plain(oo), oo, vv, 1.0);    // oovv[mn, ef]
    }
    s->stackLA.ensure(ctx, oo, ko + kv, 2);
    pack_stacked(ctx, s->stackLA, ko, Tl, plain(1), plain(oo), oo, vv, 1.0);              // Tl[ij, ef]
    // W' = oooo + X
    gett_tc_views(ctx, s->stackXW.view(0, kv), s->stackLA.view(ko, kv), oo, oo, 1.0, 1.0, s->Wp.p, plain(1),
                  plain(oo), s->oooo.p, name);
}

static void ladder_stacks_l(CCState *s, const double *Tl, const char *name) {
    Ctx *ctx = s->ctx;
    const long long o = s->o, v = s->v, oo = o * o, vv = v * v;
    const long long ko = (oo + 127) / 128 * 128, kv = (vv + 127) / 128 * 128;
    pack_stacked(ctx, s->stackLA, 0, s->Wp.p, plain(oo), plain(1), oo, oo, 1.0);          // W'[mn, ij] as (ij, mn)
    pack_stacked(ctx, s->stackLB, 0, Tl, plain(oo), plain(1), vv, oo, 1.0);               // Tl[mn, ab] as (ab, mn)
    gett_tc_views(ctx, s->stackLA.view(0, ko + kv), s->stackLB.view(0, ko + kv), oo, vv, 1.0, 1.0, s->L.p,
                  plain(1), plain(oo), s->oovv.p, name);
}

// ---------------------------------------------------------------------------------------
// The folded ladders (split precision, nocc <= 64).  The ladders' output is pair-symmetric,
// L[i,j,a,b] = L[j,i,b,a], like Tl (T2, or T2 + tau for CCSD).  For p = (i <= j), q = (a <= b)
// and s = +-1, L_s[p,q] = 1/2 (L[i,j,a,b] + s L[i,j,b,a]) is s-symmetric in (i,j) too, so
//   L[i,j,a,b] = L+[p,q] + sgn L-[p,q]   (sgn = +1 for i < j, -1 for i > j; L- = 0 for i = j or a = b),
// and every contraction over a pair (e,f) with an s-symmetric factor A_s[.,(e,f)] = Tl[.,e,f] +
// s Tl[.,f,e] runs over e <= f only: sum_ef g[ef] A_s[ef] / 2 = sum_{e<=f} A_s[ef] w_s[ef] with the
// weight w_s[ef] = 1/2 (g[ef] + s g[fe]), 1/4 g[ee] on the diagonal (pair_fold).  So
//   X_s   = Xw_s . A_s^T                       (K = the nq pairs (e <= f))
//   L_s   = O_s + [C_s | A_s] . [A_s^T | B_s]^T  (K = np pairs (m <= n), then the nq pairs (e <= f))
// with C_s the fold of W'[mn,ij] over (m,n) (hole-hole ladder), B_s that of vvvv (particle
// ladder), O_s = 1/2 oovv folded over (a,b): two GEMMs of M = np, N = nq, K = np + nq in place
// of one of M = o^2, N = v^2, K = o^2 + v^2, about a quarter of its work; X likewise halves.
// ---------------------------------------------------------------------------------------
static void pair_begin(CCState *s) {
    if (s->stackPB[0].buf.p) return;
    Ctx *ctx = s->ctx;
    const long long o = s->o, v = s->v, oo = o * o, vv = v * v, ov = o * v;
    const long long np = o * (o + 1) / 2, nq = v * (v + 1) / 2;
    const long long kp = (np + 127) / 128 * 128, kq = (nq + 127) / 128 * 128;
    {
        // B_s[(a<=b), (e<=f)] from vvvv[ab,ef] (rows a + v b, K e + v f)
        DBuf<double> tmp(ctx, (size_t)(2 * nq * nq));
        pair_fold(ctx, s->vvvv.p, nq, true, 0, 1, v, (int)v, vv, vv * v, 0.5, true, tmp.p);
        for (int k = 0; k < 2; ++k) {
            s->stackPB[k].ensure(ctx, nq, kp + kq, 2);
            pack_stacked(ctx, s->stackPB[k], kp, tmp.p + k * nq * nq, plain(1), plain(nq), nq, nq, 1.0);
        }
    }
    {
        // Xw_s[mn, (e<=f)] from oovv[mn,ef]
        DBuf<double> tmp(ctx, (size_t)(2 * oo * nq));
        pair_fold(ctx, s->oovv.p, oo, false, oo, 1, 0, (int)v, oo, oo * v, 0.5, true, tmp.p);
        for (int k = 0; k < 2; ++k) {
            s->stackPX[k].ensure(ctx, oo, kq, 2);
            pack_stacked(ctx, s->stackPX[k], 0, tmp.p + k * oo * nq, plain(1), plain(oo), oo, nq, 1.0);
        }
    }
    if (s->method == 1) {
        // Yw_s[(a,m), (e<=f)] from <am|ef> = ovvv[m,a,f,e] (row a + v m at a o + m, K at e ovv + f ov)
        DBuf<double> tmp(ctx, (size_t)(2 * ov * nq));
        pair_fold(ctx, s->ovvv.p, ov, false, v, o, 1, (int)v, ov * v, ov, 0.5, true, tmp.p);
        for (int k = 0; k < 2; ++k) {
            s->stackPY[k].ensure(ctx, ov, kq, 2);
            pack_stacked(ctx, s->stackPY[k], 0, tmp.p + k * ov * nq, plain(1), plain(ov), ov, nq, 1.0);
        }
        s->Ypm = DBuf<double>(ctx, (size_t)(2 * np * ov));
    }
    // O_s[(i<=j), (a<=b)] = 1/2 (oovv[ij,ab] + s oovv[ij,ba])
    s->Opm = DBuf<double>(ctx, (size_t)(2 * np * nq));
    pair_fold(ctx, s->oovv.p, np, true, 0, 1, o, (int)v, oo, oo * v, 0.5, false, s->Opm.p);
    s->Apm = DBuf<double>(ctx, (size_t)(2 * np * nq));
    s->Lpm = DBuf<double>(ctx, (size_t)(2 * np * nq));
    s->Cpm = DBuf<double>(ctx, (size_t)(2 * np * np));
    s->Xpm = DBuf<double>(ctx, (size_t)(2 * oo * np));
    s->invF = DBuf<double>(ctx, (size_t)(np * nq));
    inv_denominators_folded(ctx, s->eps.p, (int)o, (int)v, s->invF.p);
    for (int k = 0; k < 2; ++k) s->stackPA[k].ensure(ctx, np, kp + kq, 2);
}

// A_s from Tl, then W' = oooo + X: X[mn,ij] = X+[mn,p] + sgn X-[mn,p]
static void pair_x(CCState *s, const double *Tl, const char *name) {
    Ctx *ctx = s->ctx;
    pair_begin(s);
    const long long o = s->o, v = s->v, oo = o * o;
    const long long np = o * (o + 1) / 2, nq = v * (v + 1) / 2;
    const long long kp = (np + 127) / 128 * 128, kq = (nq + 127) / 128 * 128;
    // A_s[(i<=j), (e<=f)] = Tl[i,j,e,f] + s Tl[i,j,f,e]
    pair_fold(ctx, Tl, np, true, 0, 1, o, (int)v, oo, oo * v, 1.0, false, s->Apm.p);
    for (int k = 0; k < 2; ++k) {
        pack_stacked(ctx, s->stackPA[k], kp, s->Apm.p + k * np * nq, plain(1), plain(np), np, nq, 1.0);
        gett_tc_views(ctx, s->stackPX[k].view(0, kq), s->stackPA[k].view(kp, kq), oo, np, 1.0, 0.0,
                      s->Xpm.p + k * oo * np, plain(1), plain(oo), nullptr, name);
    }
    pair_unfold(ctx, s->Xpm.p, oo * np, s->oooo.p, (int)o, oo, oo, 1, oo, 1, false, s->Wp.p);
}

// L_s = O_s + C_s . A_s + A_s . B_s^T, C_s the fold of the finished W'
static void pair_l(CCState *s, const char *name) {
    Ctx *ctx = s->ctx;
    const long long o = s->o, v = s->v, oo = o * o;
    const long long np = o * (o + 1) / 2, nq = v * (v + 1) / 2;
    const long long kp = (np + 127) / 128 * 128, kq = (nq + 127) / 128 * 128;
    // C_s[(i<=j), (m<=n)] from W'[mn,ij] (at m + o n + o^2 (i + o j))
    pair_fold(ctx, s->Wp.p, np, true, 0, oo, oo * o, (int)o, 1, o, 0.5, true, s->Cpm.p);
    for (int k = 0; k < 2; ++k) {
        pack_stacked(ctx, s->stackPA[k], 0, s->Cpm.p + k * np * np, plain(1), plain(np), np, np, 1.0);
        pack_stacked(ctx, s->stackPB[k], 0, s->Apm.p + k * np * nq, plain(np), plain(1), nq, np, 1.0);
        gett_tc_views(ctx, s->stackPA[k].view(0, kp + kq), s->stackPB[k].view(0, kp + kq), np, nq, 1.0, 1.0,
                      s->Lpm.p + k * np * nq, plain(1), plain(np), s->Opm.p + k * np * nq, name);
    }
}

// CCSD: Y[ij,(a,m)] = ooovQ + Y+[p,(a,m)] + sgn Y-[p,(a,m)], Y_s = A_s . Yw_s^T
static void pair_y(CCState *s, double *Y, const char *name) {
    Ctx *ctx = s->ctx;
    const long long o = s->o, v = s->v, oo = o * o, ov = o * v;
    const long long np = o * (o + 1) / 2, nq = v * (v + 1) / 2;
    const long long kp = (np + 127) / 128 * 128, kq = (nq + 127) / 128 * 128;
    for (int k = 0; k < 2; ++k)
        gett_tc_views(ctx, s->stackPA[k].view(kp, kq), s->stackPY[k].view(0, kq), np, ov, 1.0, 0.0,
                      s->Ypm.p + k * np * ov, plain(1), plain(np), nullptr, name);
    pair_unfold(ctx, s->Ypm.p, np * ov, s->ooovQ.p, (int)o, ov, 1, oo, 1, np, true, Y);
}

// ---------------------------------------------------------------------------------------
// The ring contractions in split precision, on K-stacked packs (gett_tc_views).  With the
// block width kb = roundup(ov, 128) and T2 read in the ring GEMMs' two layouts,
//   R1 = T2[i,m,a,e] (rows (i,a), K (m,e)) and R23 = T2[m,i,a,e] (the same rows, m unit-stride),
// and U (CCSD: T2 + 2 tau; CCD: T2) in the R23 layout:
//   WJ  = J0 + [1/2 oovvT | -1/2 oovv] . [R1 ; U23]    (one GEMM, K = 2 ov)
//   WK  = K0 + 1/2 oovv[n,m,e,f] . U23
//   Z   = [R23 | R1] . [-WJ ; W12]                     (one GEMM, K = 2 ov)
//       + R23 (rows (i,b)) . WK (columns (a,j))
// Rows of WJ / WK are (m,e), columns (j,b); the weights are packed once (stackW).
// ---------------------------------------------------------------------------------------
static void ring_stacks_begin(CCState *s, const double *U) {
    Ctx *ctx = s->ctx;
    const long long o = s->o, v = s->v, oo = o * o, ov = o * v, oov = oo * v;
    const long long kb = (ov + 127) / 128 * 128;
    const bool ccsd = s->method == 1;
    if (!s->stackW.buf.p) {
        s->stackW.ensure(ctx, ov, 3 * kb, 2);
        const double *wt = (s->reference_df_wmbej ? s->oovv.p : s->oovvT.p);
        // [-1/2 oovv | 1/2 oovvT | 1/2 oovv']: rows (m,e), K (n,f)
        pack_stacked(ctx, s->stackW, 0, s->oovv.p, mode2(o, 1, oo), mode2(o, o, oov), ov, ov, -0.5);
        pack_stacked(ctx, s->stackW, kb, wt, mode2(o, 1, oo), mode2(o, o, oov), ov, ov, 0.5);
        pack_stacked(ctx, s->stackW, 2 * kb, s->oovv.p, mode2(o, o, oo), mode2(o, 1, oov), ov, ov, 0.5);
    }
    // CCD [R23 | R1]; CCSD [U23 | R1 | R23 | t1] (t1 as one column of a 128-wide block)
    s->stackT.ensure(ctx, ov, ccsd ? 3 * kb + 128 : 2 * kb, 2);
    pack_stacked(ctx, s->stackT, 0, U, mode2(o, o, oo), mode2(o, 1, oov), ov, ov, 1.0);        // U23 (CCD: R23)
    pack_stacked(ctx, s->stackT, kb, s->T.p, mode2(o, 1, oo), mode2(o, o, oov), ov, ov, 1.0);   // R1
    if (ccsd) {
        pack_stacked(ctx, s->stackT, 2 * kb, s->T.p, mode2(o, o, oo), mode2(o, 1, oov), ov, ov, 1.0);   // R23
        pack_stacked(ctx, s->stackT, 3 * kb, s->t1.p, plain(1), plain(1), ov, 1, 1.0);                  // t1
    }
    const Mode jb = mode2(o, ov * v, ov);
    d2d(ctx, s->WJ.p, s->ovvoJ.p, (size_t)(ov * ov));
    d2d(ctx, s->WK.p, s->ovovK.p, (size_t)(ov * ov));
    // [U23 | R1] against [-1/2 oovv | 1/2 oovvT]; U23 against 1/2 oovv[n,m,e,f]
    gett_tc_views(ctx, s->stackW.view(0, 2 * kb), s->stackT.view(0, 2 * kb), ov, ov, 1.0, 1.0, s->WJ.p, plain(1), jb,
                  nullptr, ccsd ? "ccsd_wj" : "ccd_wj");
    gett_tc_views(ctx, s->stackW.view(2 * kb, kb), s->stackT.view(0, kb), ov, ov, 1.0, 1.0, s->WK.p, plain(1), jb,
                  nullptr, ccsd ? "ccsd_wk" : "ccd_wk");
}

// Z = [R23 | R1] . [-WJ ; W12] (beta 0), then Z += R23 . WK.  CCSD also carries the rank-one
// t1[i,a] q[b,j] (the hole-hole ladder's tau F~mi terms, undone) as a third K block:
// Z = [R1 | R23 | t1] . [W12 ; -WJ ; q].
static void ring_stacks_z(CCState *s, const double *q) {
    Ctx *ctx = s->ctx;
    const long long o = s->o, v = s->v, oo = o * o, ov = o * v, oov = oo * v;
    const long long kb = (ov + 127) / 128 * 128;
    const bool ccsd = s->method == 1;
    s->stackR.ensure(ctx, ov, ccsd ? 2 * kb + 128 : 2 * kb, 2);
    pack_stacked(ctx, s->stackR, ccsd ? kb : 0, s->WJ.p, plain(ov), plain(1), ov, ov, -1.0);
    pack_stacked(ctx, s->stackR, ccsd ? 0 : kb, s->W12.p, plain(ov), plain(1), ov, ov, 1.0);
    if (ccsd) pack_stacked(ctx, s->stackR, 2 * kb, q, plain(1), plain(1), ov, 1, 1.0);
    s->stackK.ensure(ctx, ov, kb, 2);
    pack_stacked(ctx, s->stackK, 0, s->WK.p, plain(ov), plain(1), ov, ov, 1.0);
    const char *name = ccsd ? "ccsd_ring" : "ccd_ring";
    const long long kz = ccsd ? 2 * kb + 128 : 2 * kb;
    gett_tc_views(ctx, s->stackT.view(ccsd ? kb : 0, kz), s->stackR.view(0, kz), ov, ov, 1.0, 0.0, s->Z.p,
                  mode2(o, 1, oo), mode2(v, oov, o), nullptr, name);
    gett_tc_views(ctx, s->stackT.view(ccsd ? 2 * kb : 0, kb), s->stackK.view(0, kb), ov, ov, 1.0, 1.0, s->Z.p,
                  mode2(o, 1, oov), mode2(v, oo, o), nullptr, name);
}

// ---------------------------------------------------------------------------------------
// CCD sweep (FP64 or split precision for the contractions; everything else FP64)
// ---------------------------------------------------------------------------------------
double ccd_sweep(CCState *s, int prec) {
    Ctx *ctx = s->ctx;
    const long long o = s->o, v = s->v, oo = o * o, ov = o * v, oov = oo * v, vv = v * v;
    const double *T = s->T.p;
    // Every operand of this sweep is read-only once formed, so its split-precision packs can be
    // shared between the GEMMs that use it; the buffers that change from sweep to sweep lose
    // their packs here (the integrals keep theirs).
    for (const double *p : {s->T.p, s->Tn.p, s->Wp.p, s->WJ.p, s->WK.p, s->W12.p, s->Fae.p, s->Fmi.p})
        pack_cache_drop(ctx, p);
    s->cache_operands = is_split(prec);
    const double *W = s->oovv.p;

    // In split precision the ladders and the ring contractions run on K-stacked packs (two planes).
    const bool stacked = prec == JUES_PREC_SPLIT || prec == JUES_PREC_SPLIT2;
    const bool pairl = stacked && t2_finalize_folds((int)o, (int)v);   // the folded ladders
    // W'[mn,ij] = oooo[mn,ij] + X[mn,ij], X = sum_ef oovv[mn,ef] T[ij,ef]  (Wmnij + the Wabef T-part)
    if (pairl)
        pair_x(s, T, "ccd_x");
    else if (stacked)
        ladder_stacks_x(s, T, "ccd_x");
    else
        G(s, prec, "ccd_x", oo, oo, vv, 1.0, W, plain(1), plain(oo), T, plain(oo), plain(1), 1.0, s->Wp.p,
          plain(1), plain(oo), s->oooo.p);
    // Fmi[m,i] = sum_nef oovv[m,n,e,f] T~[i,n,e,f] = sum_n 2 X[mn,in] - X[mn,ni]      (RCCD.jl:216)
    fmi_from_x(ctx, s->Wp.p, s->oooo.p, (int)o, s->Fmi.p);
    // - T[i,m,a,b] Fmi[m,j] - T[m,j,a,b] Fmi[m,i] (RCCD.jl:244) as hole-hole ladder terms:
    // W'[(m,n),(i,j)] -= [m = i] Fmi[n,j] + [n = j] Fmi[m,i]
    wp_fmi(ctx, s->Wp.p, s->Fmi.p, (int)o);
    // L = oovv + (W')^T.T + T.vvvv^T                                     (RCCD.jl:243-246)
    if (pairl) {
        pair_l(s, "ccd_pp_ladder");
    } else if (stacked) {
        ladder_stacks_l(s, T, "ccd_pp_ladder");
    } else {
        G(s, prec, "ccd_hh_ladder", oo, vv, oo, 1.0, s->Wp.p, plain(oo), plain(1), T, plain(1), plain(oo),
          1.0, s->L.p, plain(1), plain(oo), W);
        G(s, prec, "ccd_pp_ladder", oo, vv, vv, 1.0, T, plain(1), plain(oo), s->vvvv.p, plain(vv), plain(1),
          1.0, s->L.p, plain(1), plain(oo), nullptr, false, true);
    }

    // Ring intermediates in (me),(bj) layout, their columns taken in (j,b) order.  With the pair
    // symmetry T[i,j,a,b] = T[j,i,b,a] and oovvT = 2 oovv[m,n,e,f] - oovv[n,m,e,f]:
    //   WmBeJ = ovvo + 1/2 oovv[m,n,e,f] T~[n,j,f,b] - 1/2 oovv[n,m,e,f] T[n,j,f,b]   (RCCD.jl:400)
    //         = ovvo + 1/2 oovvT[m,n,e,f] T[j,n,b,f] - 1/2 oovv[m,n,e,f] T[n,j,b,f]
    //   WmBEj = -ovov[m,b,j,e] + 1/2 T[j,n,f,b] oovv[n,m,e,f]                    (RCCD.jl:445)
    //         = -ovov[m,b,j,e] + 1/2 oovv[n,m,e,f] T[n,j,b,f]
    // so T enters as B in the two layouts the ring GEMMs below read it as A (one pack each) and
    // no T~ is formed.  DF-RCCD.jl:239-242 reads WmBeJ's last term as oovv[m,n,e,f] T[n,j,f,b];
    // then the first term's weights are oovv instead of oovvT.
    const Mode jb = mode2(o, ov * v, ov);   // column (j,b) of a [(m,e),(b,j)] array
    if (stacked) {
        ring_stacks_begin(s, T);
    } else {
        d2d(ctx, s->WJ.p, s->ovvoJ.p, (size_t)(ov * ov));
        d2d(ctx, s->WK.p, s->ovovK.p, (size_t)(ov * ov));
        G(s, prec, "ccd_wj", ov, ov, ov, 0.5, s->reference_df_wmbej ? W : s->oovvT.p, mode2(o, 1, oo),
          mode2(o, o, oov), T, mode2(o, o, oov), mode2(o, 1, oo), 1.0, s->WJ.p, plain(1), jb, nullptr, true);
        G(s, prec, "ccd_wj", ov, ov, ov, -0.5, W, mode2(o, 1, oo), mode2(o, o, oov), T, mode2(o, 1, oov),
          mode2(o, o, oo), 1.0, s->WJ.p, plain(1), jb, nullptr, true);
        G(s, prec, "ccd_wk", ov, ov, ov, 0.5, W, mode2(o, o, oo), mode2(o, 1, oov), T, mode2(o, 1, oov),
          mode2(o, o, oo), 1.0, s->WK.p, plain(1), jb, nullptr, true);
    }
    // W12 = 2 WJ + WK
    axpby(ctx, (size_t)(ov * ov), 2.0, s->WJ.p, 1.0, s->WK.p, s->W12.p);
    // Fae[a,e] = -sum_{mnf} T~[m,n,a,f] oovv[m,n,e,f] (RCCD.jl:179) from the traces over m of the
    // GEMM parts of WJ and WK at [(m,e),(a,m)]: -(tJ + 2 tK), or -2(tJ + tK) in the DF-RCCD.jl
    // form; then W12[(j,e),(b,j)] += Fae[b,e], so that the first ring GEMM also gives the
    // T[i,j,a,e] Fae[b,e] term of RCCD.jl:243
    fae_from_rings(ctx, s->WJ.p, s->tr0.p, s->WK.p, s->tr0.p + vv, (int)o, (int)v, s->reference_df_wmbej ? 2.0 : 1.0,
                   2.0, s->Fae.p, s->W12.p);

    // Z: the terms of RCCD.jl:243-254 whose (i,a)<->(j,b) images are added by t2_finalize
    double *Z = s->Z.p;
    if (stacked) {
        ring_stacks_z(s, nullptr);
    } else {
        // + T[i,m,a,e] (2WmBeJ + WmBEj + [m = j] Fae)[m,b,e,j]
        G(s, prec, "ccd_ring", ov, ov, ov, 1.0, T, mode2(o, 1, oo), mode2(o, o, oov), s->W12.p, plain(1),
          plain(ov), 0.0, Z, mode2(o, 1, oo), mode2(v, oov, o));
        // - T[m,i,a,e] WmBeJ[m,b,e,j]
        G(s, prec, "ccd_ring", ov, ov, ov, -1.0, T, mode2(o, o, oo), mode2(o, 1, oov), s->WJ.p, plain(1),
          plain(ov), 1.0, Z, mode2(o, 1, oo), mode2(v, oov, o));
        // + T[m,i,b,e] WmBEj[m,a,e,j]
        G(s, prec, "ccd_ring", ov, ov, ov, 1.0, T, mode2(o, o, oo), mode2(o, 1, oov), s->WK.p, plain(1),
          plain(ov), 1.0, Z, mode2(o, 1, oov), mode2(v, oo, o));
    }

    s->cache_operands = false;
    // with DIIS the step norm comes from its error vector (the same |Tn - T|^2), so the
    // finalisation skips it: two of its five FP64 operations per element
    const double *Lf = pairl ? s->Lpm.p : s->L.p, *Df = pairl ? s->invF.p : s->invD.p;
    if (s->opts.diis) {
        t2_finalize(ctx, Lf, Z, Df, (int)o, (int)v, nullptr, s->Tn.p, nullptr, nullptr, pairl);
        return -1.0;
    }
    return t2_finalize(ctx, Lf, Z, Df, (int)o, (int)v, T, s->Tn.p, nullptr, nullptr, pairl);
}

// ---------------------------------------------------------------------------------------
// DIIS (mRCCD.jl:138-208) in FP64: keep the last diis_size-1 (amplitude, error) pairs, B[k,l] =
// e_k.e_l scaled by max|B|, bordered by -1/0, c = B^-1 [0..0,-1], T = sum c_k v_k.
// ---------------------------------------------------------------------------------------
static bool solve_small(std::vector<double> A, std::vector<double> b, int n, std::vector<double> &x) {
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(A[r * n + c]) > std::fabs(A[p * n + c])) p = r;
        if (A[p * n + c] == 0.0) return false;
        if (p != c) {
            for (int k = 0; k < n; ++k) std::swap(A[c * n + k], A[p * n + k]);
            std::swap(b[c], b[p]);
        }
        for (int r = c + 1; r < n; ++r) {
            double f = A[r * n + c] / A[c * n + c];
            for (int k = c; k < n; ++k) A[r * n + k] -= f * A[c * n + k];
            b[r] -= f * b[c];
        }
    }
    x.assign(n, 0.0);
    for (int r = n - 1; r >= 0; --r) {
        double t = b[r];
        for (int k = r + 1; k < n; ++k) t -= A[r * n + k] * x[k];
        x[r] = t / A[r * n + r];
    }
    return true;
}

static void diis_reset(CCState *s) {
    s->dcount = 0;
    s->dhead = 0;
    s->dorder.clear();
    s->gram.clear();
}

// the slot of the next (amplitude, error) pair, the oldest evicted when full; olds = the stored
// errors that stay, in insertion order
static int diis_begin(CCState *s, size_t len, std::vector<const double *> &olds) {
    Ctx *ctx = s->ctx;
    const int cap = std::max(1, s->opts.diis_size - 1);
    if ((int)s->dv.size() < cap) {
        s->dv.resize(cap);
        s->de.resize(cap);
    }
    int slot;
    if (s->dcount < cap) {
        slot = s->dcount++;
    } else {
        slot = s->dorder.front();
        s->dorder.erase(s->dorder.begin());
        s->gram.erase(s->gram.begin());
        for (auto &row : s->gram) row.erase(row.begin());
    }
    if (s->dv[slot].n < len) {
        s->dv[slot] = DBuf<double>(ctx, len);
        s->de[slot] = DBuf<double>(ctx, len);
    }
    olds.resize(s->dorder.size());
    for (size_t k = 0; k < s->dorder.size(); ++k) olds[k] = s->de[s->dorder[k]].p;
    return slot;
}

// the slot's pair is stored and dots = [e.e, olds_k.e]: extend the Gram matrix, solve, and
// extrapolate into x
static void diis_finish(CCState *s, double *x, int slot, size_t len, const std::vector<double> &dots,
                        double *ee) {
    Ctx *ctx = s->ctx;
    const int m = (int)s->dorder.size() + 1;
    s->dorder.push_back(slot);
    std::vector<double> row(m);
    for (int k = 0; k < m - 1; ++k) row[k] = dots[1 + k];
    row[m - 1] = dots[0];
    if (ee) *ee = dots[0];   // |xn - x|^2
    for (int k = 0; k < m - 1; ++k) s->gram[k].push_back(row[k]);
    s->gram.push_back(row);
    double mx = 0.0;
    for (int k = 0; k < m; ++k)
        for (int l = 0; l < m; ++l) mx = std::max(mx, std::fabs(s->gram[k][l]));
    const int nb = m + 1;
    std::vector<double> B(nb * nb, -1.0), rhs(nb, 0.0), c;
    B[m * nb + m] = 0.0;
    for (int k = 0; k < m; ++k)
        for (int l = 0; l < m; ++l) B[k * nb + l] = mx > 0 ? s->gram[k][l] / mx : 0.0;
    rhs[m] = -1.0;
    if (mx == 0.0 || !solve_small(B, rhs, nb, c)) {
        d2d(ctx, x, s->dv[slot].p, len);   // degenerate subspace: plain update
        return;
    }
    std::vector<const double *> vecs(m);
    for (int k = 0; k < m; ++k) vecs[k] = s->dv[s->dorder[k]].p;
    lincomb(ctx, len, m, vecs.data(), c.data(), x);
}

// The sweep's output buffer (CCD: Tn; CCSD: Xn = [t1n | pad | Tn]) and the DIIS slot's amplitude
// buffer trade places, so that the sweep writes straight into the slot that keeps its output:
// called once before the sweep and once after it.  CCSD's views are re-pointed and its pad kept
// zero (it is part of the DIIS vector).
static void diis_swap_output(CCState *s, int slot) {
    if (s->method == 0) {
        std::swap(s->Tn, s->dv[slot]);
        return;
    }
    const size_t ov = (size_t)s->o * s->v, t2n = (size_t)s->o * s->o * s->v * s->v;
    std::swap(s->Xn, s->dv[slot]);
    s->t1n = view_of(s->Xn.p, ov);
    s->Tn = view_of(s->Xn.p + s->xoff, t2n);
    if (s->xoff > ov) fill(s->ctx, s->Xn.p + ov, s->xoff - ov, 0.0);
}

// After the sweep wrote its output xn into dv[slot] (diis_swap_output): x = the vector fed into
// the sweep (length len, device); on return x holds the extrapolated vector and *ee = |xn - x|^2.
static void diis_step(CCState *s, double *x, int slot, const std::vector<const double *> &olds, size_t len,
                      double *ee) {
    // the new error and its overlaps with the stored errors, in one pass
    std::vector<double> dots(olds.size() + 1);
    diis_error(s->ctx, len, s->dv[slot].p, x, nullptr, s->de[slot].p, (int)olds.size(), olds.data(), dots.data());
    diis_finish(s, x, slot, len, dots, ee);
}

// ---------------------------------------------------------------------------------------
// set-up
// ---------------------------------------------------------------------------------------
// validated state with its dimensions, options and orbital energies; no blocks yet
static std::unique_ptr<CCState> cc_begin(Ctx *ctx, int method, int n, int o, int v, const double *eps_dev,
                                         const jues_cc_opts &opts) {
    JUES_REQUIRE(method == 0 || method == 1, "method must be 0 (CCD) or 1 (CCSD)");
    JUES_REQUIRE(n > 0 && o > 0 && v > 0 && o + v <= n, "need 0 < nocc, 0 < nvir, nocc + nvir <= nbf");
    JUES_REQUIRE(opts.maxit >= 0, "maxit must be >= 0");
    JUES_REQUIRE(opts.diis_size >= 2 && opts.diis_size <= 16 || !opts.diis, "diis_size must be in 2..16");
    JUES_REQUIRE(valid_precision(opts.precision), "unknown precision");
    JUES_REQUIRE(opts.guess >= 0 && opts.guess <= 2, "unknown guess");
    std::unique_ptr<CCState> s(new CCState());
    s->ctx = ctx;
    s->method = method;
    s->n = n; s->o = o; s->v = v;
    s->opts = opts;
    s->precision = opts.precision;
    s->eps = DBuf<double>(ctx, n);
    d2d(ctx, s->eps.p, eps_dev, n);
    return s;
}

// ring seeds, work arrays, the initial amplitudes and their energy
static CCState *cc_finish(std::unique_ptr<CCState> s) {
    Ctx *ctx = s->ctx;
    const int method = s->method, o = s->o, v = s->v;
    const jues_cc_opts &opts = s->opts;
    const long long oo = (long long)o * o, vv = (long long)v * v, ov = (long long)o * v;
    const size_t t2n = (size_t)(oo * vv);
    // ring seeds in (me),(bj) layout: ovvoJ[(me),(bj)] = ovvo[m,b,e,j] (CCD) or, for CCSD,
    // the same value read from oovv[m,j,e,b] (= <mj|eb> = (me|jb), as mRCCSD.jl:187 does);
    // ovovK[(me),(bj)] = -ovov[m,b,j,e]
    s->ovvoJ = DBuf<double>(ctx, (size_t)(ov * ov));
    s->ovovK = DBuf<double>(ctx, (size_t)(ov * ov));
    {
        if (method == 0) {
            // box (m, e, b, j); ovvo[m,b,e,j] offset m + o b + ov e + ovv j
            Perm4 p{{o, v, v, o}, {1, ov, o, ov * v}, {1, o, ov, ov * v}};
            permute4(ctx, p, 1.0, s->ovvo.p, 0.0, s->ovvoJ.p);
        } else {
            // box (m, e, b, j); oovv[m,j,e,b] offset m + o j + oo e + oov b
            Perm4 p{{o, v, v, o}, {1, oo, oo * v, o}, {1, o, ov, ov * v}};
            permute4(ctx, p, 1.0, s->oovv.p, 0.0, s->ovvoJ.p);
        }
        // ovov[m,b,j,e] offset m + o b + ov j + ovo e
        Perm4 q{{o, v, v, o}, {1, ov * o, o, ov}, {1, o, ov, ov * v}};
        permute4(ctx, q, -1.0, s->ovov.p, 0.0, s->ovovK.p);
    }
    s->tr0 = DBuf<double>(ctx, (size_t)(2 * vv));
    ring_traces(ctx, s->ovvoJ.p, nullptr, s->ovovK.p, nullptr, o, v, s->tr0.p, s->tr0.p + vv);
    s->oovvT = DBuf<double>(ctx, t2n);
    t_tilde(ctx, s->oovv.p, o, v, s->oovvT.p);
    if (method == 1) {
        // ooovT[m,n,i,e] = 2 ooov[m,n,i,e] - ooov[n,m,i,e]; c1, c2 = the ooov diagonal sums
        const size_t n3 = (size_t)(oo * ov);
        s->ooovT = DBuf<double>(ctx, n3);
        DBuf<double> sw(ctx, n3);
        Perm4 p{{o, o, o, v}, {o, 1, oo, oo * o}, {1, o, oo, oo * o}};
        permute4(ctx, p, 1.0, s->ooov.p, 0.0, sw.p);
        axpby(ctx, n3, 2.0, s->ooov.p, -1.0, sw.p, s->ooovT.p);
        s->c12 = DBuf<double>(ctx, (size_t)(3 * ov));
        ooov_diag_sums(ctx, s->ooov.p, o, v, s->c12.p);
        // box (i, j, a, m): ooov[m,i,j,a] at m + o i + oo j + ooo a; ooovQ[i,j,a,m] at i + o j + oo a + oov m
        s->ooovQ = DBuf<double>(ctx, n3);
        Perm4 q{{o, o, v, o}, {o, oo, oo * o, 1}, {1, o, oo, oo * v}};
        permute4(ctx, q, 1.0, s->ooov.p, 0.0, s->ooovQ.p);
        // M1[(i,a),(m,e)] = 2 oovv[i,m,a,e] - ovov[m,a,i,e], box (i, a, m, e)
        s->M1 = DBuf<double>(ctx, (size_t)(ov * ov));
        Perm4 p1{{o, v, o, v}, {1, oo, o, oo * v}, {1, o, ov, ov * o}};
        permute4(ctx, p1, 2.0, s->oovv.p, 0.0, s->M1.p);
        Perm4 p2{{o, v, o, v}, {ov, o, 1, ov * o}, {1, o, ov, ov * o}};
        permute4(ctx, p2, -1.0, s->ovov.p, 1.0, s->M1.p);
    }
    s->invD = DBuf<double>(ctx, t2n);
    inv_denominators(ctx, s->eps.p, o, v, s->invD.p);
    if (method == 1) {
        // [t1 | pad | T2] contiguous for DIIS, T2 16-byte aligned; the pad stays zero
        s->xoff = (size_t)(ov + 1) / 2 * 2;
        s->X = DBuf<double>(ctx, s->xoff + t2n);
        s->Xn = DBuf<double>(ctx, s->xoff + t2n);
        fill(ctx, s->X.p, s->xoff, 0.0);
        fill(ctx, s->Xn.p, s->xoff, 0.0);
        s->t1 = view_of(s->X.p, (size_t)ov);
        s->T = view_of(s->X.p + s->xoff, t2n);
        s->t1n = view_of(s->Xn.p, (size_t)ov);
        s->Tn = view_of(s->Xn.p + s->xoff, t2n);
    } else {
        s->T = DBuf<double>(ctx, t2n);
        s->Tn = DBuf<double>(ctx, t2n);
    }
    if (method == 1) s->Tt = DBuf<double>(ctx, t2n);   // the CCD sweep forms no T~
    s->Z = DBuf<double>(ctx, t2n);
    s->L = DBuf<double>(ctx, t2n);
    s->Wp = DBuf<double>(ctx, (size_t)(oo * oo));
    s->WJ = DBuf<double>(ctx, (size_t)(ov * ov));
    s->WK = DBuf<double>(ctx, (size_t)(ov * ov));
    s->W12 = DBuf<double>(ctx, (size_t)(ov * ov));
    s->Fae = DBuf<double>(ctx, (size_t)vv);
    s->Fmi = DBuf<double>(ctx, (size_t)oo);
    if (method == 1) {
        s->Fme = DBuf<double>(ctx, (size_t)ov);
        s->U = DBuf<double>(ctx, t2n);
        s->Fmt = DBuf<double>(ctx, (size_t)oo);
        s->fwork = DBuf<double>(ctx, (size_t)(4 * vv + ov));
        fill(ctx, s->t1.p, (size_t)ov, 0.0);
    }
    // initial amplitudes
    if (method == 1 || opts.guess == JUES_GUESS_MP2) {
        divide_by_d(ctx, s->oovv.p, s->eps.p, o, v, s->T.p);   // mRCCSD.jl:66
    } else if (opts.guess == JUES_GUESS_ZERO) {
        fill(ctx, s->T.p, t2n, 0.0);                          // mRCCD.jl:245
    } else {
        // RCCD.jl:145-160: T[i,j,a,b] = ovov[i,a,j,b] / D
        Perm4 p{{o, o, v, v}, {1, ov, o, ov * o}, {1, o, oo, oo * v}};
        permute4(ctx, p, 1.0, s->ovov.p, 0.0, s->Tn.p);
        divide_by_d(ctx, s->Tn.p, s->eps.p, o, v, s->T.p);
    }
    s->energy = cc_total_energy(s.get());
    s->e_prev = s->energy;
    diis_reset(s.get());
    ctx->check_flags();
    return s.release();
}


CCState *cc_create(Ctx *ctx, int method, const double *g, int n, const double *Cocc, int o,
                   const double *Cvir, int v, const double *eps_dev, const jues_cc_opts &opts) {
    std::unique_ptr<CCState> s = cc_begin(ctx, method, n, o, v, eps_dev, opts);
    const long long oo = (long long)o * o, vv = (long long)v * v, ov = (long long)o * v;
    const size_t t2n = (size_t)(oo * vv);
    // integral blocks (mRCCD.jl:120-127, mRCCSD.jl:102-110), physicists' notation
    const int iprec = opts.transform_precision >= 0 ? opts.transform_precision : opts.precision;
    s->oovv = DBuf<double>(ctx, t2n);
    s->ovov = DBuf<double>(ctx, t2n);
    s->oooo = DBuf<double>(ctx, (size_t)(oo * oo));
    s->vvvv = DBuf<double>(ctx, (size_t)(vv * vv));
    Ctx::HostPhase ph_blocks(ctx, "host:integral_blocks");
    // the blocks share their common quarter steps (the occupied blocks' first quarter)
    std::vector<std::pair<std::string, double *>> blocks = {
        {"OOVV", s->oovv.p}, {"OVOV", s->ovov.p}, {"OOOO", s->oooo.p}, {"VVVV", s->vvvv.p}};
    if (method == 0) {
        s->ovvo = DBuf<double>(ctx, t2n);
        blocks.push_back({"OVVO", s->ovvo.p});
    } else {
        s->ooov = DBuf<double>(ctx, (size_t)(oo * ov));
        s->ovvv = DBuf<double>(ctx, (size_t)(ov * vv));
        blocks.push_back({"ooov", s->ooov.p});
        blocks.push_back({"ovvv", s->ovvv.p});
    }
    get_eri_blocks(ctx, iprec, g, n, Cocc, o, Cvir, v, blocks, true, 0, true);
    pack_cache_drop(ctx, g);
    return cc_finish(std::move(s));
}

CCState *cc_create_df(Ctx *ctx, const double *b, int n, int naux, const double *Cocc, int o, const double *Cvir, int v,
                      const double *eps_dev, const jues_cc_opts &opts, bool reference_wmbej) {
    JUES_REQUIRE(naux > 0, "naux must be positive");
    std::unique_ptr<CCState> s = cc_begin(ctx, 0, n, o, v, eps_dev, opts);
    s->reference_df_wmbej = reference_wmbej;
    const long long oo = (long long)o * o, vv = (long long)v * v;
    const size_t t2n = (size_t)(oo * vv);
    // DF-RCCD.jl:78-89: the four MO factors, then the five blocks the sweep reads, each once
    const int iprec = opts.transform_precision >= 0 ? opts.transform_precision : opts.precision;
    {
        DfFactors f = df_factors(ctx, iprec, b, n, naux, Cocc, o, Cvir, v, true);
        s->oovv = DBuf<double>(ctx, t2n);
        s->ovov = DBuf<double>(ctx, t2n);
        s->ovvo = DBuf<double>(ctx, t2n);
        s->oooo = DBuf<double>(ctx, (size_t)(oo * oo));
        s->vvvv = DBuf<double>(ctx, (size_t)(vv * vv));
        df_blocks(ctx, iprec, f, s->oovv.p, s->ovov.p, s->ovvo.p, s->oooo.p, s->vvvv.p);
    }
    pack_cache_clear(ctx);
    return cc_finish(std::move(s));
}

double cc_total_energy(CCState *s) {
    // CCD (RCCD.jl:99-117): E = sum oovv[i,j,a,b] (2T[i,j,a,b] - T[j,i,a,b])
    //                         = sum T[i,j,a,b] (2 oovv[i,j,a,b] - oovv[j,i,a,b]) (i <-> j in the second
    // term), one dot product with weights formed once
    if (s->method == 0 && s->oovvT.p)
        return dot(s->ctx, (size_t)s->o * s->o * s->v * s->v, s->T.p, s->oovvT.p);
    double e;
    if (s->method == 1 && s->oovvT.p) {
        // CCSD: sum oovv (2X - X^T) with X = T2 + t1 (x) t1 = T2 . oovvT + sum_ia t1[i,a] F[i,a],
        // F[i,a] = sum_jb oovvT[i,j,a,b] t1[j,b] (one GEMV into the Fme work array)
        const long long o = s->o, v = s->v, oo = o * o, ov = o * v, oov = oo * v;
        G(s, JUES_PREC_FP64, "ccenergy", ov, 1, ov, 1.0, s->oovvT.p, mode2(o, 1, oo), mode2(o, o, oov), s->t1.p,
          plain(1), plain(0), 0.0, s->Fme.p, plain(1), plain(0), nullptr, true, false);
        e = dot(s->ctx, (size_t)(oo * v * v), s->T.p, s->oovvT.p) + dot(s->ctx, (size_t)ov, s->t1.p, s->Fme.p);
    } else {
        e = cc_energy(s->ctx, s->oovv.p, s->T.p, s->method == 1 ? s->t1.p : nullptr, s->o, s->v);
    }
    if (s->fock && s->method == 1) e += 2.0 * dot(s->ctx, (size_t)s->o * s->v, s->fOV.p, s->t1.p);   // AutoRCCSD.jl:43
    return e;
}

CCState *cc_create_auto(Ctx *ctx, const double *g, const double *h, int n, const double *C, int nmo, int ndocc,
                        int fcn, const jues_cc_opts &opts) {
    JUES_REQUIRE(n > 0 && nmo > 0 && nmo <= n, "need 0 < nmo <= nbf");
    JUES_REQUIRE(ndocc > 0 && ndocc < nmo, "need 0 < ndocc < nmo");
    JUES_REQUIRE(fcn >= 0 && fcn < ndocc, "need 0 <= fcn < ndocc");
    const int o = ndocc - fcn, v = nmo - ndocc;
    // Fock matrix of the orbitals (all ndocc occupied define the density), AutoRCCSD.jl:218-233
    DBuf<double> f(ctx, (size_t)nmo * nmo);
    get_fock(ctx, g, h, n, C, nmo, C, ndocc, f.p);
    std::vector<double> hf((size_t)nmo * nmo);
    JUES_CHECK_CUDA(cudaMemcpyAsync(hf.data(), f.p, hf.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    JUES_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    auto F = [&](int p, int q) { return hf[(size_t)p + (size_t)nmo * q]; };
    // eps has nbf entries like the orbital energies it replaces (the sweeps read the first o + v)
    std::vector<double> eps((size_t)n, 0.0), foo((size_t)o * o), fov((size_t)o * v), fvv((size_t)v * v);
    for (int i = 0; i < o; ++i) eps[i] = F(fcn + i, fcn + i);
    for (int a = 0; a < v; ++a) eps[o + a] = F(ndocc + a, ndocc + a);
    for (int i = 0; i < o; ++i)
        for (int j = 0; j < o; ++j) foo[i + (size_t)o * j] = i == j ? 0.0 : F(fcn + i, fcn + j);
    for (int i = 0; i < o; ++i)
        for (int a = 0; a < v; ++a) fov[i + (size_t)o * a] = F(fcn + i, ndocc + a);
    for (int a = 0; a < v; ++a)
        for (int b = 0; b < v; ++b) fvv[a + (size_t)v * b] = a == b ? 0.0 : F(ndocc + a, ndocc + b);
    DBuf<double> deps(ctx, eps.size());
    JUES_CHECK_CUDA(cudaMemcpyAsync(deps.p, eps.data(), eps.size() * sizeof(double), cudaMemcpyHostToDevice,
                                    ctx->stream));
    // the active orbitals are column ranges of C: occupied fcn..ndocc-1, virtual ndocc..nmo-1
    jues_cc_opts op = opts;
    op.guess = JUES_GUESS_MP2;
    std::unique_ptr<CCState> s(cc_create(ctx, 1, g, n, C + (size_t)n * fcn, o, C + (size_t)n * ndocc, v, deps.p, op));
    auto up = [&](DBuf<double> &d, const std::vector<double> &hsrc) {
        d = DBuf<double>(ctx, hsrc.size());
        JUES_CHECK_CUDA(cudaMemcpyAsync(d.p, hsrc.data(), hsrc.size() * sizeof(double), cudaMemcpyHostToDevice,
                                        ctx->stream));
    };
    up(s->fOO, foo);
    up(s->fOV, fov);
    up(s->fVV, fvv);
    s->fock = true;
    s->auto_rms = true;
    // T1 = f_ov / d (AutoRCCSD.jl:253), T2 = <ij|ab>/D already set
    d2d(ctx, s->t1n.p, s->fOV.p, (size_t)o * v);
    fill(ctx, s->t1.p, (size_t)o * v, 0.0);
    t1_finalize(ctx, s->t1n.p, s->eps.p, o, v, s->t1.p);
    d2d(ctx, s->t1.p, s->t1n.p, (size_t)o * v);
    s->energy = cc_total_energy(s.get());
    s->e_prev = s->energy;
    ctx->check_flags();
    return s.release();
}

// amplitude vector for DIIS: CCD = T2; CCSD = [t1 | pad | T2] (the X buffer)
static void cc_one(CCState *s, int prec) {
    Ctx *ctx = s->ctx;
    const size_t t2n = (size_t)s->o * s->o * s->v * s->v;
    cudaEvent_t e0, e1;
    JUES_CHECK_CUDA(cudaEventCreate(&e0));
    JUES_CHECK_CUDA(cudaEventCreate(&e1));
    JUES_CHECK_CUDA(cudaEventRecord(e0, ctx->stream));
    double r2;
    // with DIIS the sweep's output goes straight into the slot that keeps it
    int slot = -1;
    std::vector<const double *> olds;
    const size_t dlen = s->method == 0 ? t2n : s->xoff + t2n;
    if (s->opts.diis) {
        slot = diis_begin(s, dlen, olds);
        diis_swap_output(s, slot);
    }
    if (s->method == 0) {
        r2 = ccd_sweep(s, prec);
    } else {
        r2 = ccsd_sweep(s, prec);
    }
    if (s->opts.diis) {
        diis_swap_output(s, slot);
        double ee = 0.0;
        diis_step(s, s->method == 0 ? s->T.p : s->X.p, slot, olds, dlen, &ee);
        if (r2 < 0.0) r2 = ee;   // the sweep left the step norm to DIIS
    } else {
        std::swap(s->T, s->Tn);
        if (s->method == 1) {
            std::swap(s->t1, s->t1n);
            std::swap(s->X, s->Xn);
        }
    }
    double rn = std::sqrt(r2);
    s->e_prev = s->energy;
    s->energy = cc_total_energy(s);
    if (s->auto_rms) {
        const double n1 = (double)s->o * s->v, n2 = n1 * n1;
        rn = std::max(std::sqrt(s->r1sq) / n1, std::sqrt(s->r2sq) / n2);
    }
    JUES_CHECK_CUDA(cudaEventRecord(e1, ctx->stream));
    JUES_CHECK_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->check_flags();
    if (!std::isfinite(s->energy) || !std::isfinite(rn))
        throw Error(JUES_ENONFINITE, "CC iterations produced a non-finite energy or step (diverged)");
    s->iters += 1;
    jues_iter_log rec;
    rec.iter = s->iters;
    rec.precision = prec;
    rec.energy = s->energy;
    rec.rnorm = rn;
    rec.ms = ms;
    s->log.push_back(rec);
}

static bool cc_converged(const CCState *s) {
    if (s->log.empty()) return false;
    const jues_iter_log &r = s->log.back();
    bool any = false, ok = true;
    if (s->opts.r_conv > 0) { any = true; ok = ok && r.rnorm < s->opts.r_conv; }
    if (s->opts.e_conv > 0) { any = true; ok = ok && std::fabs(s->energy - s->e_prev) < s->opts.e_conv; }
    return any && ok;
}

// Split precision stops improving once the step reaches the BF16-split noise floor; detect
// that (no decrease over two sweeps after it fell below 1e-5) and hand over to FP64 sweeps.
static bool at_noise_floor(const CCState *s) {
    const auto &L = s->log;
    if (L.size() < 3) return false;
    const double a = L[L.size() - 3].rnorm, b = L[L.size() - 2].rnorm, c = L.back().rnorm;
    return c < 1e-5 && c > 0.5 * b && b > 0.5 * a;
}

void cc_iterate(CCState *s, int nsweeps, int *done, int *converged) {
    int k = 0;
    bool conv = false;
    const bool split = is_split(s->precision);
    while (k < nsweeps) {
        const int prec = (split && s->refine_left >= 0) ? JUES_PREC_FP64 : s->precision;
        cc_one(s, prec);
        ++k;
        conv = cc_converged(s);
        if (split && s->opts.refine > 0) {
            if (s->refine_left < 0) {
                if (conv || at_noise_floor(s)) {
                    // hand over to the closing FP64 sweeps; restart DIIS with exact residuals
                    s->refine_left = s->opts.refine;
                    diis_reset(s);
                    conv = false;
                }
                continue;
            }
            if (--s->refine_left == 0) break;
        }
        if (conv) break;
    }
    s->converged = conv;
    if (done) *done = k;
    if (converged) *converged = conv ? 1 : 0;
}

void cc_amplitudes(CCState *s, double *t1_host, double *t2_host) {
    Ctx *ctx = s->ctx;
    const size_t t2n = (size_t)s->o * s->o * s->v * s->v;
    if (t2_host)
        JUES_CHECK_CUDA(cudaMemcpyAsync(t2_host, s->T.p, t2n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (t1_host) {
        if (s->method == 1)
            JUES_CHECK_CUDA(cudaMemcpyAsync(t1_host, s->t1.p, (size_t)s->o * s->v * sizeof(double),
                                            cudaMemcpyDeviceToHost, ctx->stream));
        else
            std::memset(t1_host, 0, (size_t)s->o * s->v * sizeof(double));
    }
    ctx->sync();
}

double CCState::sweep_flops(int prec) const {
    (void)prec;
    return ccd_sweep_flops(o, v);
}

}  // namespace jues

namespace jues {

// ---------------------------------------------------------------------------------------
// CCSD sweep (RCCSD.jl:150-289 on the six blocks of mRCCSD.jl:102-110).
// Work buffers: aux1 = Ttau = T2 + tau, U = T2 + 2 tau (tau = t1 (x) t1, never stored); aux2 =
// the o^3 v intermediates.  Rewrites, exact given the pair symmetry T2[i,j,a,b] = T2[j,i,b,a]:
//   * Wabef is never formed: its vvvv part is the particle ladder on the resident (cached)
//     vvvv, its t1 parts go through Y[ij,a,m] = sum_ef Ttau[ij,ef] <am|ef>:
//       sum_ef Ttau[ij,ef] (-t1[m,b] <am|ef> - t1[m,a] <mb|ef>) = -sum_m t1[m,b] Y[ij,a,m] - (image),
//     the image being added by the finalisation (Z[i,j,a,b] + Z[j,i,b,a]);
//   * the T2 parts of WmBeJ / WmBEj are three GEMMs: 1/2 oovvT[m,n,e,f] T2[j,n,b,f] and
//     -1/2 oovv[m,n,e,f] U[n,j,b,f] into WJ, 1/2 oovv[n,m,e,f] U[n,j,b,f] into WK, with T2 and
//     U in the layouts the ring GEMMs read them in;
//   * Fmi's T2 part is the trace of X = oovv . Ttau^T (the hole-hole intermediate), Fae's T2
//     and t1 parts are traces of WJ and WK (ccsd_fae_kernel), T1's <ma|fe> terms traces of Y;
//   * the F~ae term rides in the first ring GEMM (W12[(j,e),(b,j)] += F~ae[b,e]) and the F~mi
//     terms in the hole-hole ladder (W'[(m,n),(i,j)] -= [m = i] F~mi[n,j] + [n = j] F~mi[m,i]),
//     whose Ttau in place of T2 the finalisation undoes with the rank-one t1[i,a] q[b,j],
//     q[b,j] = sum_m t1[m,b] F~mi[m,j], and its image.
// Every contraction runs in the sweep's precision; the split engine keeps the ones with a
// dimension below 16 in FP64 by itself.
// ---------------------------------------------------------------------------------------
double ccsd_sweep(CCState *s, int prec) {
    Ctx *ctx = s->ctx;
    const long long o = s->o, v = s->v, oo = o * o, ov = o * v, oov = oo * v, ooo = oo * o,
                    vv = v * v, ovv = ov * v;
    const size_t t2n = (size_t)(oo * vv);
    const double *T = s->T.p, *t1 = s->t1.p, *W = s->oovv.p, *ooov = s->ooov.p, *ovvv = s->ovvv.p,
                 *ovov = s->ovov.p;
    if (s->aux1.n < t2n) s->aux1 = DBuf<double>(ctx, t2n);
    if (s->aux2.n < (size_t)(ooo * v)) s->aux2 = DBuf<double>(ctx, (size_t)(ooo * v));
    double *Ttau = s->aux1.p, *U = s->U.p;
    double *tGJ = s->fwork.p, *tGK = tGJ + vv, *H1 = tGK + vv, *G2 = H1 + vv, *q = G2 + vv;
    // T2, Ttau and U are read-only in this sweep: their packs are shared between the GEMMs that
    // read them in the same layout (the ladders, X and Y; WJ, WK and the rings)
    for (const double *p : {(const double *)s->T.p, (const double *)s->Tn.p, (const double *)Ttau, (const double *)U})
        pack_cache_drop(ctx, p);
    ccsd_tau(ctx, T, t1, (int)o, (int)v, Ttau, U);

    // Fme = sum_nf oovvT[m,n,e,f] t1[n,f] (RCCSD.jl:204-210)
    G(s, JUES_PREC_FP64, "ccsd_fme", ov, 1, ov, 1.0, s->oovvT.p, mode2(o, 1, oo), mode2(o, o, oov), t1, plain(1),
      plain(0), 0.0, s->Fme.p, plain(1), plain(0), nullptr, true, false);
    // In split precision the ladders, Y and the ring contractions run on K-stacked packs.
    const bool stacked = prec == JUES_PREC_SPLIT || prec == JUES_PREC_SPLIT2;   // two planes
    const bool pairl = stacked && t2_finalize_folds((int)o, (int)v);             // the folded ladders
    // W' = oooo + X, X = sum_ef oovv[mn,ef] Ttau[ij,ef] (Wmnij and Wabef's T2 + tau parts)
    if (pairl)
        pair_x(s, Ttau, "ccsd_x");
    else if (stacked)
        ladder_stacks_x(s, Ttau, "ccsd_x");
    else
        G(s, prec, "ccsd_x", oo, oo, vv, 1.0, W, plain(1), plain(oo), Ttau, plain(oo), plain(1), 1.0, s->Wp.p,
          plain(1), plain(oo), s->oooo.p, true, true);
    // Fmi (RCCSD.jl:195-203): sum_nef oovv[m,n,e,f] (2 Ts[i,n,e,f] - Ts[n,i,e,f]), Ts = T2 + tau/2,
    // = the trace of X less 1/2 Fme[m,e] t1[i,e]; then the ooov t1 terms
    fmi_from_x(ctx, s->Wp.p, s->oooo.p, (int)o, s->Fmi.p);
    G(s, JUES_PREC_FP64, "ccsd_fmi", o, o, v, -0.5, s->Fme.p, plain(1), plain(o), t1, plain(o), plain(1), 1.0,
      s->Fmi.p, plain(1), plain(o));
    G(s, prec, "ccsd_fmi_t1", oo, 1, ov, 2.0, ooov, mode2(o, 1, oo), mode2(o, o, ooo), t1,
      plain(1), plain(0), 1.0, s->Fmi.p, plain(1), plain(0), nullptr, true, false);
    G(s, prec, "ccsd_fmi_t1", oo, 1, ov, -1.0, ooov, mode2(o, o, oo), mode2(o, 1, ooo), t1,
      plain(1), plain(0), 1.0, s->Fmi.p, plain(1), plain(0), nullptr, true, false);
    // W' += t1[j,e] ooov[m,n,i,e] + t1[i,e] ooov[n,m,j,e]
    G(s, prec, "ccsd_wmnij_t1", ooo, o, v, 1.0, ooov, plain(1), plain(ooo), t1, plain(o),
      plain(1), 1.0, s->Wp.p, plain(1), plain(ooo), nullptr, true, false);
    G(s, prec, "ccsd_wmnij_t1", ooo, o, v, 1.0, ooov, plain(1), plain(ooo), t1, plain(o),
      plain(1), 1.0, s->Wp.p, mode3(o, o, o, 1, ooo), plain(oo), nullptr, true, false);
    if (s->fock) {
        // non-canonical Fock terms: Fmi += f_mi + 1/2 t1[i,e] f_me, Fme += f_me (Fae's are in
        // ccsd_fae_kernel; the diagonals of f_oo and f_vv are zero, they sit in the resolvents)
        axpby(ctx, (size_t)oo, 1.0, s->fOO.p, 1.0, s->Fmi.p, s->Fmi.p);
        G(s, prec, "ccsd_fock", o, o, v, 0.5, s->fOV.p, plain(1), plain(o), t1, plain(o), plain(1),
          1.0, s->Fmi.p, plain(1), plain(o));
        axpby(ctx, (size_t)ov, 1.0, s->fOV.p, 1.0, s->Fme.p, s->Fme.p);
    }
    // F~mi[m,j] = Fmi + 1/2 Fme[m,e] t1[j,e], into the hole-hole ladder
    d2d(ctx, s->Fmt.p, s->Fmi.p, (size_t)oo);
    G(s, JUES_PREC_FP64, "ccsd_ftilde", o, o, v, 0.5, s->Fme.p, plain(1), plain(o), t1, plain(o), plain(1), 1.0,
      s->Fmt.p, plain(1), plain(o));
    wp_fmi(ctx, s->Wp.p, s->Fmt.p, (int)o);
    // L = oovv + W'^T Ttau + Ttau vvvv^T  (Wabef's t1 parts go through Y below)
    if (pairl) {
        pair_l(s, "ccsd_pp_ladder");
    } else if (stacked) {
        ladder_stacks_l(s, Ttau, "ccsd_pp_ladder");
    } else {
        G(s, prec, "ccsd_hh_ladder", oo, vv, oo, 1.0, s->Wp.p, plain(oo), plain(1), Ttau, plain(1), plain(oo),
          1.0, s->L.p, plain(1), plain(oo), W, false, true);
        G(s, prec, "ccsd_pp_ladder", oo, vv, vv, 1.0, Ttau, plain(1), plain(oo), s->vvvv.p, plain(vv),
          plain(1), 1.0, s->L.p, plain(1), plain(oo), nullptr, true, true);
    }

    // ring intermediates (RCCSD.jl:229-247), layout [(m,e),(b,j)], columns taken in (j,b) order
    const Mode jb = mode2(o, ov * v, ov);
    if (stacked) {
        ring_stacks_begin(s, U);
    } else {
        d2d(ctx, s->WJ.p, s->ovvoJ.p, (size_t)(ov * ov));
        d2d(ctx, s->WK.p, s->ovovK.p, (size_t)(ov * ov));
        G(s, prec, "ccsd_wj", ov, ov, ov, 0.5, s->oovvT.p, mode2(o, 1, oo), mode2(o, o, oov), T, mode2(o, o, oov),
          mode2(o, 1, oo), 1.0, s->WJ.p, plain(1), jb, nullptr, true, true);
        G(s, prec, "ccsd_wj", ov, ov, ov, -0.5, W, mode2(o, 1, oo), mode2(o, o, oov), U, mode2(o, 1, oov),
          mode2(o, o, oo), 1.0, s->WJ.p, plain(1), jb, nullptr, true, true);
        G(s, prec, "ccsd_wk", ov, ov, ov, 0.5, W, mode2(o, o, oo), mode2(o, 1, oov), U, mode2(o, 1, oov),
          mode2(o, o, oo), 1.0, s->WK.p, plain(1), jb, nullptr, true, true);
    }
    ring_traces(ctx, s->WJ.p, s->tr0.p, s->WK.p, s->tr0.p + vv, (int)o, (int)v, tGJ, tGK);
    // the t1 terms: WJ += t1[j,f] <mb|ef> - t1[n,b] <mn|ej>, WK += -t1[j,f] <mb|fe> + t1[n,b] <nm|ej>
    G(s, prec, "ccsd_wj_t1", ovv, o, v, 1.0, ovvv, mode3(o, v, 1, ov, o), plain(ovv), t1,
      plain(o), plain(1), 1.0, s->WJ.p, mode3(o, v, 1, o, ov), plain(ovv), nullptr, true, false);
    G(s, prec, "ccsd_wj_t1", ov * o, v, o, -1.0, ooov, mode3(o, v, o, ooo, oo), plain(1), t1,
      plain(1), plain(o), 1.0, s->WJ.p, mode3(o, v, 1, o, ovv), plain(ov), nullptr, true, false);
    G(s, prec, "ccsd_wk_t1", ovv, o, v, -1.0, ovvv, mode3(o, v, 1, ovv, o), plain(ov), t1,
      plain(o), plain(1), 1.0, s->WK.p, mode3(o, v, 1, o, ov), plain(ovv), nullptr, true, false);
    G(s, prec, "ccsd_wk_t1", ov * o, v, o, 1.0, ooov, mode3(o, v, 1, ooo, oo), plain(o), t1,
      plain(1), plain(o), 1.0, s->WK.p, mode3(o, v, 1, o, ovv), plain(ov), nullptr, true, false);
    axpby(ctx, (size_t)(ov * ov), 2.0, s->WJ.p, 1.0, s->WK.p, s->W12.p);
    // Fae (the exchange t1 term as RCCSD.jl:190 or mRCCSD.jl:140), H1, G2; W12 += [m = j] F~ae
    ccsd_fae(ctx, s->WJ.p, s->tr0.p, s->WK.p, s->tr0.p + vv, tGJ, tGK, t1, s->c12.p, s->Fme.p,
             s->fock ? s->fOV.p : nullptr, s->fock ? s->fVV.p : nullptr, (int)o, (int)v,
             s->opts.ccsd_fae == JUES_CCSD_FAE_MRCCSD, s->Fae.p, H1, G2, s->W12.p);

    // Y[ij,(a,m)] = sum_ef Ttau[i,j,e,f] <am|ef> (<am|ef> = ovvv[m,a,f,e])
    double *Y = s->aux2.p;
    if (pairl) {
        pair_y(s, Y, "ccsd_y");
    } else if (stacked) {
        // Ttau[ij,ef] from the ladder stack; ovvv as (a,m) x (e,f), packed once
        const long long ko = (oo + 127) / 128 * 128, kv = (vv + 127) / 128 * 128;
        if (!s->stackY.buf.p) {
            s->stackY.ensure(ctx, ov, kv, 2);
            pack_stacked(ctx, s->stackY, 0, ovvv, mode2(v, o, 1), mode2(v, ovv, ov), ov, vv, 1.0);
        }
        gett_tc_views(ctx, s->stackLA.view(ko, kv), s->stackY.view(0, kv), oo, ov, 1.0, 1.0, Y, plain(1), plain(oo),
                      s->ooovQ.p, "ccsd_y");
    } else {
        G(s, prec, "ccsd_y", oo, ov, vv, 1.0, Ttau, plain(1), plain(oo), ovvv, mode2(v, ovv, ov), mode2(v, o, 1),
          1.0, Y, plain(1), plain(oo), s->ooovQ.p, true, true);
    }

    // T1 (RCCSD.jl:248-259) into t1n
    double *R1 = s->t1n.p;
    G(s, prec, "ccsd_t1", o, v, v, 1.0, t1, plain(1), plain(o), s->Fae.p, plain(v), plain(1),
      0.0, R1, plain(1), plain(o));
    G(s, prec, "ccsd_t1", o, v, o, -1.0, s->Fmi.p, plain(o), plain(1), t1, plain(1), plain(o),
      1.0, R1, plain(1), plain(o));
    // Fme[m,e] (2 T2[i,m,a,e] - T2[m,i,a,e]), one read of T2
    if (stacked) {
        // sum_me (2 T2[i,m,a,e] - T2[m,i,a,e]) Fme[m,e] = [R1 | R23] . [2 Fme ; -Fme] on the ring packs
        const long long kb = (ov + 127) / 128 * 128;
        s->stackF.ensure(ctx, 1, 2 * kb, 2);
        pack_stacked(ctx, s->stackF, 0, s->Fme.p, plain(0), plain(1), 1, ov, 2.0);
        pack_stacked(ctx, s->stackF, kb, s->Fme.p, plain(0), plain(1), 1, ov, -1.0);
        gett_tc_views(ctx, s->stackT.view(kb, 2 * kb), s->stackF.view(0, 2 * kb), ov, 1, 1.0, 1.0, R1, plain(1),
                      plain(ov), nullptr, "ccsd_t1");
    } else {
        t1_fme(ctx, T, s->Fme.p, (int)o, (int)v, R1);
    }
    // t1[m,e] (2 <im|ae> - <ma|ie>) through M1, formed once
    G(s, prec, "ccsd_t1", ov, 1, ov, 1.0, s->M1.p, plain(1), plain(ov), t1, plain(1), plain(0), 1.0, R1, plain(1),
      plain(0), nullptr, true, false);
    // - sum_mne T2[m,n,a,e] (2 <mn|ie> - <nm|ie>)
    G(s, prec, "ccsd_t1_ooov", o, v, oov, -1.0, s->ooovT.p, plain(oo), mode2(oo, 1, ooo), T,
      mode2(oo, 1, oov), plain(oo), 1.0, R1, plain(1), plain(o), nullptr, true, false);
    // the <ma|fe> terms from Y (its ooov seed's traces, c2 and c3, taken off)
    t1_ytrace(ctx, Y, t1, G2, H1, s->c12.p, (int)o, (int)v, R1);

    // Z's t1 terms with t1 on b, by their (i,a)<->(j,b) images all of the form
    // -sum_m Q[i,j,a,m] t1[m,b], with Q (in place of Y, layout [(i,j),(a,m)]) =
    //   Y[i,j,a,m]                                 (Wabef's t1 parts)
    // + <mi|ja> = ooov[m,i,j,a]                            (- t1[m,a] <mb|ij>, imaged; Y's seed)
    // + Y1[j,m,i,a], Y1[i,m,j,b] = sum_e t1[i,e] <mj|eb>   (- tau[i,m,e,a] <mb|ej>, imaged)
    // + Y2[i,m,a,j], Y2[i,m,a,j] = sum_e t1[i,e] <ma|je>   (- tau[i,m,e,b] <am|ej>)
    G(s, prec, "ccsd_z_tau", o, oov, v, 1.0, t1, plain(1), plain(o), W, plain(oo), mode3(o, o, 1, o, oov), 1.0, Y,
      plain(o), mode3(o, o, oov, 1, oo), nullptr, false, true);
    G(s, prec, "ccsd_z_tau", o, oov, v, 1.0, t1, plain(1), plain(o), ovov, plain(oov), plain(1), 1.0, Y, plain(1),
      mode3(o, v, oov, oo, o), nullptr, false, true);

    // q[b,j] = sum_m t1[m,b] F~mi[m,j]: the hole-hole ladder's tau[i,m,a,b] F~mi[m,j] terms, undone by
    // the rank-one t1[i,a] q[b,j] (and its image): a K block of the stacked ring GEMM, or a term of
    // the finalisation
    G(s, JUES_PREC_FP64, "ccsd_q", v, o, o, 1.0, t1, plain(o), plain(1), s->Fmt.p, plain(1), plain(o), 0.0, q,
      plain(1), plain(v));

    // Z (RCCSD.jl:264-284, one member of each (i,a)<->(j,b) pair)
    double *Z = s->Z.p;
    // + T2[i,m,a,e] (2 WmBeJ + WmBEj + [m = j] F~ae)[m,b,e,j] - T2[m,i,a,e] WmBeJ[m,b,e,j]
    // + T2[m,i,b,e] WmBEj[m,a,e,j]
    if (stacked) {
        ring_stacks_z(s, q);
    } else {
        G(s, prec, "ccsd_ring", ov, ov, ov, 1.0, T, mode2(o, 1, oo), mode2(o, o, oov), s->W12.p, plain(1),
          plain(ov), 0.0, Z, mode2(o, 1, oo), mode2(v, oov, o), nullptr, true, false);
        G(s, prec, "ccsd_ring", ov, ov, ov, -1.0, T, mode2(o, o, oo), mode2(o, 1, oov), s->WJ.p, plain(1),
          plain(ov), 1.0, Z, mode2(o, 1, oo), mode2(v, oov, o), nullptr, true, false);
        G(s, prec, "ccsd_ring", ov, ov, ov, 1.0, T, mode2(o, o, oo), mode2(o, 1, oov), s->WK.p, plain(1),
          plain(ov), 1.0, Z, mode2(o, 1, oov), mode2(v, oo, o), nullptr, true, false);
    }
    // Z[i,j,a,b] -= sum_m Q[i,j,a,m] t1[m,b]: Wabef's t1 parts and the tau and ooov t1 terms
    G(s, prec, "ccsd_y_t1", oov, v, o, -1.0, Y, plain(1), plain(oov), t1, plain(1), plain(o), 1.0, Z,
      plain(1), plain(oov));
    // + t1[i,e] <ab|ej> = t1[i,e] ovvv[j,a,b,e]
    G(s, prec, "ccsd_z_ovvv", o, ovv, v, 1.0, t1, plain(1), plain(o), ovvv, plain(ovv), plain(1), 1.0, Z,
      plain(1), plain(o), nullptr, false, true);

    if (s->fock) axpby(ctx, (size_t)ov, 1.0, s->fOV.p, 1.0, R1, R1);   // + f_ia
    // with DIIS the step norm comes from its error vector over [t1 | T2] (the same squared sum), so
    // the finalisation skips it unless the per-block norms are wanted (AutoRCCSD's rms)
    const bool norms = !s->opts.diis || s->auto_rms;
    double r2 = t2_finalize(ctx, pairl ? s->Lpm.p : s->L.p, Z, pairl ? s->invF.p : s->invD.p, (int)o, (int)v,
                            norms ? T : nullptr, s->Tn.p, stacked ? nullptr : t1, stacked ? nullptr : q, pairl);
    // t1n = R1 / D_ia and its step norm
    const double r1 = t1_finalize(ctx, R1, s->eps.p, (int)o, (int)v, norms ? t1 : nullptr);
    if (!norms) return -1.0;
    s->r1sq = r1;
    s->r2sq = r2;
    return r2 + r1;
}

}  // namespace jues
