#pragma once
#include <vector>

#include "common.cuh"

namespace jues {

// Device-resident closed-shell CC problem (CCD or CCSD).
struct CCState {
    Ctx *ctx = nullptr;
    int method = 0;   // 0 CCD, 1 CCSD
    int n = 0, o = 0, v = 0;
    jues_cc_opts opts{};
    int precision = JUES_PREC_FP64;
    // integrals, physicists' notation, column-major as the reference's get_eri blocks
    DBuf<double> eps, oovv, ovov, ovvo, oooo, vvvv, ooov, ovvv;
    DBuf<double> invD;           // 1 / D[i,j,a,b], formed once
    DBuf<double> oovvT;          // 2 oovv[i,j,a,b] - oovv[j,i,a,b], formed once (CCD energy weights,
                                 // ring and Fme weights)
    DBuf<double> ooovT, c12;     // CCSD: 2 ooov[m,n,i,e] - ooov[n,m,i,e]; the ooov diagonal sums c1, c2, c3
    DBuf<double> ooovQ;          // CCSD: ooov[m,i,j,a] at [(i,j),(a,m)], the seed of Y
    DBuf<double> M1;             // CCSD: 2 oovv[i,m,a,e] - ovov[m,a,i,e] at [(i,a),(m,e)] (T1's t1 terms)
    DBuf<double> ovvoJ, ovovK;   // ring-intermediate seeds in (me),(bj) layout
    DBuf<double> tr0;            // their traces sum_m [(m,e),(a,m)], v x v each (trJ0 | trK0)
    // amplitudes and work arrays
    DBuf<double> T, Tn, Tt, Z, L, Wp, WJ, WK, W12, Fae, Fmi;
    DBuf<double> t1, t1n, Fme, U, Fmt;      // CCSD: U = T2 + 2 tau, Fmt = F~mi
    // CCSD: the amplitudes [t1 | pad | T2] and the sweep's output in one buffer each (the DIIS
    // vectors); t1, T and t1n, Tn are views into them, T2 starting at element xoff (even)
    DBuf<double> X, Xn;
    size_t xoff = 0;
    DBuf<double> fwork;                     // CCSD: ring traces tGJ, tGK, H1, G2 (v x v each), q (v x o)
    DBuf<double> aux1, aux2;                // CCSD scratch
    // split precision: K-stacked packs of the ring contractions.  stackW (constant, built once):
    // the WmBeJ / WmBEj weights [a | b | 1/2 oovv[n,m,e,f]] with (a, b) = (-1/2 oovv, 1/2 oovvT)
    // (CCD) or (1/2 oovvT, -1/2 oovv) (CCSD); stackT: T2[m,i,a,e] | T2[i,m,a,e] (| U[m,i,a,e],
    // CCSD); stackR: -WJ | W12; stackK: WK
    StackedPack stackW, stackT, stackR, stackK;
    // split precision: the two ladders as one GEMM, L = oovv + [W'^T | T] . [T ; vvvv]^T over
    // K = (m,n) then (e,f): stackLA = [W'^T | T] (rows (i,j)), stackLB = [T | vvvv] (rows (a,b),
    // vvvv packed once); stackXW = oovv (rows (m,n), K (e,f)) for X; stackY = ovvv as (a,m) x (e,f)
    // for CCSD's Y
    StackedPack stackLA, stackLB, stackXW, stackY;
    // split precision with nocc <= 64 (t2_finalize_folds): the same contractions folded by the pair
    // symmetry over occupied pairs p = (i <= j) (np of them) and virtual pairs q = (a <= b) (nq),
    // sign s = +1 (index 0) and -1 (index 1):
    //   A_s[p,q(e,f)] = Tl[i,j,e,f] + s Tl[i,j,f,e]                     (Apm, per sweep)
    //   X_s[mn,p]  = sum_q Xw_s[mn,q] A_s[p,q]                            (X = X+ + sgn X-)
    //   L_s[p,q]   = O_s[p,q] + sum_p' C_s[p,p'] A_s[p',q] + sum_q' A_s[p,q'] B_s[q,q']
    //   Y_s[p,am]  = sum_q A_s[p,q] Yw_s[am,q]                            (CCSD)
    // with the weights B_s (vvvv), Xw_s (oovv), Yw_s (ovvv) and C_s (W', per sweep) folded over
    // their contracted pair at 1/2 (1/4 on its diagonal), and O_s = 1/2 oovv folded over (a, b).
    // stackPA[s] = [C_s | A_s] (rows p), stackPB[s] = [A_s^T | B_s] (rows q, B_s packed once),
    // stackPX[s] = Xw_s (rows (m,n)), stackPY[s] = Yw_s (rows (a,m)).
    DBuf<double> Apm, Cpm, Lpm, Opm, Xpm, Ypm;
    DBuf<double> invF;           // the folded 1/D, np x nq (the finalisation of the folded form)
    StackedPack stackPA[2], stackPB[2], stackPX[2], stackPY[2];
    // CCSD, split precision: [2 Fme | -Fme] (one row, K = the ring blocks R1 and R23 of stackT),
    // so T1's T2.Fme terms are one GEMM on T2's ring packs
    StackedPack stackF;
    // DIIS (FP64): amplitude vectors and their errors, ring buffer of diis_size-1 pairs
    std::vector<DBuf<double>> dv, de;
    std::vector<std::vector<double>> gram;   // gram[k][l] = e_k . e_l, k,l in insertion order
    int dcount = 0;     // pairs stored
    int dhead = 0;      // next slot
    std::vector<int> dorder;   // slots in insertion order
    double energy = 0.0, e_prev = 0.0;
    int iters = 0;
    int refine_left = -1;          // split precision: closing FP64 sweeps left (-1 = not started)
    bool cache_operands = false;   // keep split packs of every sweep operand (CCD)
    bool converged = false;
    bool reference_df_wmbej = false;   // DF-RCCD.jl's index order in WmBeJ's last term
    // general (non-canonical) Fock matrix, AutoRCCSD.jl: off-diagonal occupied and virtual
    // blocks and the occupied-virtual block; eps then holds the Fock diagonal
    bool fock = false;
    DBuf<double> fOO, fOV, fVV;
    bool auto_rms = false;       // rnorm = max(||dT1||/len(T1), ||dT2||/len(T2)) (AutoRCCSD.jl:172-174)
    double r1sq = 0.0, r2sq = 0.0;   // squared step norms of the last sweep
    std::vector<jues_iter_log> log;
    double sweep_flops(int prec) const;
};

CCState *cc_create(Ctx *ctx, int method, const double *gao_dev, int n, const double *Cocc_dev, int o,
                   const double *Cvir_dev, int v, const double *eps_dev, const jues_cc_opts &opts);
// CCD on density-fitted integrals: b[mu,nu,Q] (device, n x n x naux) is the fitted factor
// (DF-RCCD.jl:11-54); the five blocks are built from its MO factors and kept resident
CCState *cc_create_df(Ctx *ctx, const double *b, int n, int naux, const double *Cocc_dev, int o,
                      const double *Cvir_dev, int v, const double *eps_dev, const jues_cc_opts &opts,
                      bool reference_wmbej);
// CCSD from a general Fock matrix, AutoRCCSD.do_rccsd (AutoRCCSD.jl:193-300): f = get_fock of
// the orbitals C (n x nmo; the first ndocc occupied), fcn frozen core orbitals, T1 = f_ov/d,
// T2 = <ij|ab>/D, per-element rms convergence
CCState *cc_create_auto(Ctx *ctx, const double *gao_dev, const double *hao_dev, int n, const double *C_dev, int nmo,
                        int ndocc, int fcn, const jues_cc_opts &opts);
double cc_total_energy(CCState *s);   // CC energy including 2 f_ov . t1 when a Fock matrix is set
void cc_iterate(CCState *s, int nsweeps, int *done, int *converged);
void cc_amplitudes(CCState *s, double *t1_host, double *t2_host);
// one CCD / CCSD sweep: Tn from T (and t1n from t1), returns the squared step norm
double ccd_sweep(CCState *s, int prec);
double ccsd_sweep(CCState *s, int prec);
// flop counts
double ccd_sweep_flops(int o, int v);
double ccd_reference_flops(int o, int v);   // mRCCD.jl GEMM set (Wabef formed)

}  // namespace jues
