#pragma once
#include "common.cuh"

namespace jues {

// Density-fitted three-index factors, all column-major on the device.
//
// b[mu,nu,Q] is the fitted AO factor: (mu nu|lam sig) ~ sum_Q b[mu,nu,Q] b[lam,sig,Q]
// (src/Backend/DF.jl:52-57 forms it as pqP Jpqh).

// b = pqP Jpqh (pqP: n x n x naux, Jpqh: naux x naux); returns a new buffer
DBuf<double> df_fit(Ctx *ctx, int prec, const double *pqP, int n, int naux, const double *Jpqh);

// out[p,q,Q] = sum_{mu,nu} C1[mu,p] b[mu,nu,Q] C2[nu,q]  (d1 x d2 x naux), the MO factors of
// DF-RMP2.jl:17-22 and DF-RCCD.jl:78-89
void df_mo_factor(Ctx *ctx, int prec, const double *b, int n, int naux, const double *C1, int d1, const double *C2,
                  int d2, double *out);

// MO factors of a closed-shell reference: boo (o x o), bov (o x v), bvo (v x o), bvv (v x v),
// each x naux.  Any pointer may be null to skip that factor.
struct DfFactors {
    int o = 0, v = 0, naux = 0;
    DBuf<double> boo, bov, bvo, bvv;
};
DfFactors df_factors(Ctx *ctx, int prec, const double *b, int n, int naux, const double *Cocc, int o,
                     const double *Cvir, int v, bool need_oo_vv);

// physicists'-notation blocks from the factors, the same numbers as get_eri's blocks of the
// fitted integrals: oovv[i,j,a,b] = (ia|jb), ovov[i,a,j,b] = (ij|ab), ovvo[i,a,b,j] = (ib|aj),
// oooo[i,j,k,l] = (ik|jl), vvvv[a,b,c,d] = (ac|bd).  Null outputs are skipped.
void df_blocks(Ctx *ctx, int prec, const DfFactors &f, double *oovv, double *ovov, double *ovvo, double *oooo,
               double *vvvv);

}  // namespace jues
