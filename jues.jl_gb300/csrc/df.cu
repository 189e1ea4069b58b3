// Density-fitted integral factors and blocks (src/Backend/DF.jl, DF-RMP2.jl, DF-RCCD.jl).
//
// Every step is one GETT over composite modes, so nothing is permuted: the MO factor is two
// quarter steps (C1 over mu, then C2 over nu, with Q riding along as part of a composite
// mode), and each four-index block is one contraction over Q whose output modes scatter it
// straight into physicists' order.
#include "df.cuh"

namespace jues {

DBuf<double> df_fit(Ctx *ctx, int prec, const double *pqP, int n, int naux, const double *Jpqh) {
    const long long nn = (long long)n * n;
    DBuf<double> b(ctx, (size_t)(nn * naux));
    GettArgs a;
    a.M = nn; a.N = naux; a.K = naux;
    a.alpha = 1.0; a.beta = 0.0;
    a.A = pqP; a.mA = plain(1); a.kA = plain(nn);
    a.B = Jpqh; a.kB = plain(1); a.nB = plain(naux);
    a.C = b.p; a.mC = plain(1); a.nC = plain(nn);
    gett(ctx, integral_precision(prec), a, "df_fit");
    return b;
}

void df_mo_factor(Ctx *ctx, int prec, const double *b, int n, int naux, const double *C1, int d1, const double *C2,
                  int d2, double *out) {
    // half[p,nu,Q] = sum_mu C1[mu,p] b[mu,nu,Q]
    DBuf<double> half(ctx, (size_t)d1 * n * naux);
    {
        GettArgs a;
        a.M = d1; a.N = (long long)n * naux; a.K = n;
        a.alpha = 1.0; a.beta = 0.0;
        a.A = C1; a.mA = plain(n); a.kA = plain(1);
        a.B = b; a.kB = plain(1); a.nB = plain(n);
        a.C = half.p; a.mC = plain(1); a.nC = plain(d1);
        gett(ctx, integral_precision(prec), a, "df_half");
    }
    // out[p,q,Q] = sum_nu half[p,nu,Q] C2[nu,q]; rows are the composite (p,Q)
    {
        GettArgs a;
        a.M = (long long)d1 * naux; a.N = d2; a.K = n;
        a.alpha = 1.0; a.beta = 0.0;
        a.A = half.p; a.mA = mode2(d1, 1, (long long)d1 * n); a.kA = plain(d1);
        a.B = C2; a.kB = plain(1); a.nB = plain(n);
        a.C = out; a.mC = mode2(d1, 1, (long long)d1 * d2); a.nC = plain(d1);
        gett(ctx, integral_precision(prec), a, "df_half");
    }
}

DfFactors df_factors(Ctx *ctx, int prec, const double *b, int n, int naux, const double *Cocc, int o,
                     const double *Cvir, int v, bool need_oo_vv) {
    DfFactors f;
    f.o = o; f.v = v; f.naux = naux;
    const size_t ov = (size_t)o * v;
    f.bov = DBuf<double>(ctx, ov * naux);
    df_mo_factor(ctx, prec, b, n, naux, Cocc, o, Cvir, v, f.bov.p);
    if (need_oo_vv) {
        // DF-RCCD.jl:82-87 forms all four; bvo is a separate transform (equal to bov^T only
        // when b is symmetric in mu, nu)
        f.bvo = DBuf<double>(ctx, ov * naux);
        f.boo = DBuf<double>(ctx, (size_t)o * o * naux);
        f.bvv = DBuf<double>(ctx, (size_t)v * v * naux);
        df_mo_factor(ctx, prec, b, n, naux, Cvir, v, Cocc, o, f.bvo.p);
        df_mo_factor(ctx, prec, b, n, naux, Cocc, o, Cocc, o, f.boo.p);
        df_mo_factor(ctx, prec, b, n, naux, Cvir, v, Cvir, v, f.bvv.p);
    }
    return f;
}

namespace {
// out = sum_Q X[(r),Q] Y[(c),Q] with X's rows r = p + dp q and Y's rows c = s + ds t, scattered
// through the output modes (rows by mC over (p,q), columns by nC over (s,t))
void contract_q(Ctx *ctx, int prec, const double *X, long long xr, const double *Y, long long yr, long long naux,
                const Mode &mC, const Mode &nC, double *out, const char *name) {
    GettArgs a;
    a.M = xr; a.N = yr; a.K = naux;
    a.alpha = 1.0; a.beta = 0.0;
    a.A = X; a.mA = plain(1); a.kA = plain(xr);
    a.B = Y; a.kB = plain(yr); a.nB = plain(1);
    a.C = out; a.mC = mC; a.nC = nC;
    gett(ctx, integral_precision(prec), a, name);
}
}  // namespace

void df_blocks(Ctx *ctx, int prec, const DfFactors &f, double *oovv, double *ovov, double *ovvo, double *oooo,
               double *vvvv) {
    const long long o = f.o, v = f.v, Q = f.naux;
    const long long oo = o * o, ov = o * v, vv = v * v;
    if (oovv)   // oovv[i,j,a,b] = sum_Q bov[i,a,Q] bov[j,b,Q]; rows (i,a), columns (j,b)
        contract_q(ctx, prec, f.bov.p, ov, f.bov.p, ov, Q, mode2(o, 1, oo), mode2(o, o, oo * v), oovv, "df_oovv");
    if (ovov)   // ovov[i,a,j,b] = sum_Q boo[i,j,Q] bvv[a,b,Q]; rows (i,j), columns (a,b)
        contract_q(ctx, prec, f.boo.p, oo, f.bvv.p, vv, Q, mode2(o, 1, ov), mode2(v, o, ov * o), ovov, "df_ovov");
    if (ovvo)   // ovvo[i,a,b,j] = sum_Q bov[i,b,Q] bvo[a,j,Q]; rows (i,b), columns (a,j)
        contract_q(ctx, prec, f.bov.p, ov, f.bvo.p, ov, Q, mode2(o, 1, ov), mode2(v, o, ov * v), ovvo, "df_ovvo");
    if (oooo)   // oooo[i,j,k,l] = sum_Q boo[i,k,Q] boo[j,l,Q]; rows (i,k), columns (j,l)
        contract_q(ctx, prec, f.boo.p, oo, f.boo.p, oo, Q, mode2(o, 1, oo), mode2(o, o, oo * o), oooo, "df_oooo");
    if (vvvv)   // vvvv[a,b,c,d] = sum_Q bvv[a,c,Q] bvv[b,d,Q]; rows (a,c), columns (b,d)
        contract_q(ctx, prec, f.bvv.p, vv, f.bvv.p, vv, Q, mode2(v, 1, vv), mode2(v, v, vv * v), vvvv, "df_vvvv");
}

}  // namespace jues
