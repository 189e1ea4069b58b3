/*
 * jues_gpu.h -- C ABI of libjuesgpu.so, the GB300 (sm_103a) implementation of the
 * JuES correlated-method hot path: AO->MO four-index transformation, closed-shell
 * MP2 energy and closed-shell CCD / CCSD amplitude iterations.
 *
 * Conventions (shared by every entry point):
 *  - All arrays are column-major (Julia layout): element X[i,j,a,b] of a d1 x d2 x d3 x d4
 *    array sits at offset i + d1*(j + d2*(a + d3*b)).  Julia arrays can be passed as is.
 *  - Pointers are host pointers unless the name ends in _dev; inputs are borrowed for the
 *    duration of the call and never modified; outputs are caller-allocated.
 *  - Every function returns 0 (JUES_OK) or a positive JUES_E* code; jues_last_error()
 *    gives the message of the last failure on the calling thread.
 *  - A jues_ctx owns one CUDA stream and every device buffer it allocates.  A context is
 *    single-threaded; different contexts may be used concurrently.  Calls are synchronous
 *    at return.
 *  - Host input arrays of 64 MB and more are page-locked in 512 MB pieces for the duration
 *    of their copy and released before the call returns (arrays the caller has already
 *    page-locked are copied as they are).  The batched entry points instead copy through a
 *    page-locked staging ring owned by the context (host threads, 3 x 64 MB).
 *
 * Reference interfaces replaced (paths within mdav2/JuES.jl):
 *  jues_tei_transform  <- JuES.Transformation.tei_transform        src/Backend/Transformation.jl:15-20,39-93
 *  jues_get_eri        <- JuES.IntegralTransformation.get_eri      src/Backend/IntegralTransformation.jl:38-101
 *  jues_rmp2           <- JuES.MollerPlesset.do_rmp2               src/MollerPlesset/RMP2.jl:11-45
 *  jues_rccd           <- JuES.CoupledCluster.{mRCCD,RCCD}.do_rccd src/CoupledCluster/mRCCD.jl:38-118, RCCD.jl:33-83
 *  jues_rccsd          <- JuES.CoupledCluster.{RCCSD,mRCCSD}.do_rccsd  src/CoupledCluster/RCCSD.jl:33-116, mRCCSD.jl:35-101
 */
#ifndef JUES_GPU_H
#define JUES_GPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define JUES_API __attribute__((visibility("default")))
#else
#define JUES_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define JUES_OK 0
#define JUES_EINVAL 1      /* bad argument (dimension, pointer, spec string, option) */
#define JUES_ENOMEM 2      /* device allocation failed or over the context's memory cap */
#define JUES_ECUDA 3       /* CUDA runtime / driver error */
#define JUES_ENOTCONV 4    /* CC iterations hit maxit before the requested convergence */
#define JUES_ENONFINITE 5  /* a NaN or Inf was found in inputs or iterates */
#define JUES_ETIMEOUT 6    /* a bounded device-side wait expired (kernel returned early) */
#define JUES_ENODEV 7      /* no usable sm_103 device */

/* Arithmetic used for the bulk of the contractions.  The split forms run on the tcgen05 tensor
 * cores (kind::f16) with FP32 accumulation: every FP64 operand is cut into 10-bit integer digits
 * ("planes") carried exactly in FP16, with a power-of-two scale per 128-wide K chunk of a row.
 * Two planes (hi + lo, three products) keep ~2^-20 relative; three (hi + mid + lo, six products)
 * keep ~2^-24, the FP32 rounding of the chunk sums. */
#define JUES_PREC_FP64 0       /* plain FP64 (the drop-in form)                                   */
#define JUES_PREC_SPLIT 1      /* the split form at <= 1 uEh: three planes for every contraction
                                  that produces integrals (four-index transforms, get_eri blocks,
                                  DF factors, the MP2 adjoint's back-transforms), two planes for
                                  the CC sweeps, jues_gemm and (T)                               */
#define JUES_PREC_SPLIT_BF16 JUES_PREC_SPLIT   /* earlier name of JUES_PREC_SPLIT              */
#define JUES_PREC_SPLIT3 2     /* three planes for every contraction                              */
#define JUES_PREC_SPLIT2 3     /* two planes for every contraction, integrals included: fastest,
                                  ~5e-6 Eh MP2 error at nbf=200 (opt-in)                          */

/* CC initial amplitudes */
#define JUES_GUESS_ZERO 0  /* T2 = 0 (mRCCD.jl:239-256); first sweep gives MP2 amplitudes   */
#define JUES_GUESS_MP2 1   /* T2 = <ij|ab>/D (mRCCSD.jl:66)                                  */
#define JUES_GUESS_OVOV 2  /* T2 = (ij|ab)/D (RCCD.jl:145-160)                               */

/* CCSD: the t1 term of Fae.  The reference's two CCSD forms differ there: RCCSD.jl:190 (and the
 * textbook closed-shell equations) contract t1[m,f] with <ma|ef>, mRCCSD.jl:140 with <me|af>. */
#define JUES_CCSD_FAE_RCCSD 0   /* <ma|ef>, RCCSD.jl:190                                        */
#define JUES_CCSD_FAE_MRCCSD 1  /* <me|af>, mRCCSD.jl:140                                       */

/* DF-RCCD equation variants */
#define JUES_DF_REFERENCE 0  /* as DF-RCCD.jl: WmBeJ's last term reads (me|nf) T[n,j,f,b]     */
#define JUES_DF_RCCD      1  /* as RCCD.jl on the fitted integrals: (ne|mf) T[n,j,f,b]         */

typedef struct jues_ctx jues_ctx;
typedef struct jues_cc jues_cc;

typedef struct {
    int maxit;        /* maximum sweeps (reference default 40)                            */
    double e_conv;    /* |E_k - E_{k-1}| threshold; <= 0 disables                          */
    double r_conv;    /* ||T_new - T_old||_2 threshold (mRCCD.jl:106); <= 0 disables        */
    int diis;         /* 0 = plain Jacobi sweeps, 1 = DIIS (mRCCD.jl:138-208, FP64)         */
    int diis_size;    /* number of stored amplitude vectors (reference max_diis = 6)        */
    int precision;    /* JUES_PREC_*                                                       */
    int guess;        /* JUES_GUESS_*                                                      */
    int refine;       /* split precision only: number of closing FP64 sweeps               */
    int transform_precision; /* precision of the integral transform; -1 = same as precision
                                (JUES_PREC_SPLIT then means three-plane integrals)            */
    int ccsd_fae;     /* CCSD only: JUES_CCSD_FAE_* (default JUES_CCSD_FAE_RCCSD)            */
} jues_cc_opts;

typedef struct {
    int iter;         /* 1-based sweep number                                            */
    int precision;    /* precision that sweep ran in                                     */
    double energy;    /* correlation energy of the amplitudes carried to the next sweep  */
    double rnorm;     /* ||T_new - T_old||_2 of the un-extrapolated update               */
    double ms;        /* device time of the sweep (CUDA events on the context stream)    */
} jues_iter_log;

/* ---- context ---------------------------------------------------------------------- */
JUES_API int jues_version(void);
JUES_API int jues_last_error(char *buf, size_t len);
JUES_API int jues_ctx_create(int device, jues_ctx **out);
/* AO integrals read in place (no reference counterpart).  Where the device reads pageable host
 * memory through the host page tables (ATS, e.g. Grace-Blackwell over NVLink-C2C), the split
 * forms pack the caller's n^4 AO array straight from host memory instead of copying it to the
 * device first.  Off by default (environment JUES_AO_DIRECT=1 turns the default on): on GB300
 * with Grace the in-place reads measured ~8 GB/s, below the page-locked copy the library uses
 * otherwise (~200 GB/s).  *active (may be NULL) tells whether it is on. */
JUES_API int jues_ctx_set_ao_direct(jues_ctx *ctx, int enable, int *active);
JUES_API int jues_ctx_destroy(jues_ctx *ctx);
/* Cap the device memory the context may hold (bytes, 0 = no cap); used to exercise the
 * out-of-memory path without exhausting the GPU. */
JUES_API int jues_ctx_set_mem_limit(jues_ctx *ctx, size_t bytes);
/* Per-kernel CUDA-event timing of the named hot kernels (0 = off). */
JUES_API int jues_ctx_set_profiling(jues_ctx *ctx, int on);
/* Total time and launch count recorded for kernels whose name starts with `prefix`. */
JUES_API int jues_ctx_profile(jues_ctx *ctx, const char *prefix, double *total_ms, long long *launches);
JUES_API int jues_ctx_profile_reset(jues_ctx *ctx);
/* Number of kernels this context has launched so far. */
JUES_API long long jues_ctx_launch_count(jues_ctx *ctx);

/* ---- dense contraction -----------------------------------------------------------------
 * C = alpha * op(A) op(B) + beta * C, column-major, op = transpose when trans != 0: the
 * BLAS.gemm! call the reference's explicit-GEMM CC (src/CoupledCluster/mRCCD.jl:274-485)
 * is built from, run by the same engine as every contraction here (FP64 or split BF16). */
JUES_API int jues_gemm(jues_ctx *ctx, int transA, int transB, int M, int N, int K, double alpha,
                       const double *A, int lda, const double *B, int ldb, double beta,
                       double *C, int ldc, int precision);

/* Allocation-free variant of jues_gemm's split-precision path.  No counterpart in the
 * reference.  For callers that cannot let the library allocate device memory when they
 * contract: host frameworks that reserve the GPU's memory at start-up and hand it out from their
 * own pool (a cudaMalloc from inside the library would fail, or escape their accounting), and
 * long-running or fixed-budget services that must not grow their device footprint after
 * start-up.  A, B and C are DEVICE pointers (column-major, C = alpha op(A) op(B) + beta C,
 * two-plane split arithmetic; K = 0 gives C = beta C); the call allocates nothing: the packed
 * operands go to a static device array of 64 MiB that every GPU loading the library holds until
 * the process exits.  Problems whose packed operands,
 * 4 (Mpad + Npad) Kpad + 4 ceil(Kpad/128) (Mpad + Npad) bytes with Mpad, Npad and Kpad rounded
 * up to 128, 128 and 64, exceed it are rejected with JUES_EINVAL.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress, with that device current).  All
 * calls share the one array and each call rewrites every byte of it that it reads: calls whose
 * execution overlaps on the GPU (other streams, other contexts on the same device) race on it.
 * Runs on the context's stream and is synchronous at return (it reads the device error flags). */
JUES_API int jues_gemm_noalloc(jues_ctx *ctx, int transA, int transB, int M, int N, int K, double alpha,
                               const double *A_dev, int lda, const double *B_dev, int ldb, double beta,
                               double *C_dev, int ldc);

/* Failure-path check: runs one device wait on a barrier phase that nothing completes, with the
 * same bounded wait as the split GEMM's pipeline.  The wait gives up after its limit (~2 s), the
 * kernel returns with the timeout flag set, and the call returns JUES_ETIMEOUT; the context stays
 * usable.  Nothing faults or hangs. */
JUES_API int jues_debug_expired_wait(jues_ctx *ctx);

/* ---- four-index transformation -------------------------------------------------------
 * out[i,a,j,b] = sum C1[mu,i] C2[nu,a] C3[lam,j] C4[sig,b] gao[mu,nu,lam,sig]
 * (chemists' (C1 C2|C3 C4)); gao is n^4, Ck is n x dk, out is d1 x d2 x d3 x d4.
 * Replaces Transformation.jl:39-93 (the 2-argument form :15-20 is C1=C2=C3=C4). */
JUES_API int jues_tei_transform(jues_ctx *ctx, const double *gao, int n,
                       const double *C1, int d1, const double *C2, int d2,
                       const double *C3, int d3, const double *C4, int d4,
                       int precision, double *out);

/* get_eri(wfn, spec; notation, fcn) for a closed-shell Wfn: spec is 4 chars of o/O/v/V
 * (lower = beta = alpha blocks for a restricted Wfn); phys != 0 selects physicists'
 * notation (IntegralTransformation.jl:46-48,96-98); fcn drops the first fcn occupied
 * columns (:54-59).  out has the block's shape in the requested notation. */
JUES_API int jues_get_eri(jues_ctx *ctx, const double *gao, int n,
                 const double *Cocc, int o, const double *Cvir, int v,
                 const char *spec, int phys, int fcn, int precision, double *out);

/* ---- MP2 -------------------------------------------------------------------------------
 * E = sum <ij|ab>(2<ij|ab> - <ij|ba>)/(e_i+e_j-e_a-e_b) (RMP2.jl:27-41). eps has n entries,
 * occupied first.  Optional k_out (o*o*v*v, may be NULL) receives <ij|ab>. */
JUES_API int jues_rmp2(jues_ctx *ctx, const double *gao, int n,
              const double *Cocc, int o, const double *Cvir, int v,
              const double *eps, int precision, double *e_out, double *k_out);

/* Density-fitted MP2 (src/MollerPlesset/DF-RMP2.jl:1-46) on the outputs of setup_df
 * (src/Backend/DF.jl:30-51): pqP[mu,nu,P] (n x n x naux, column-major) and Jpqh = J^-1/2
 * (naux x naux).  b[mu,nu,Q] = pqP Jpqh (skipped when Jpqh is NULL: pqP is then already b),
 * B[i,a,Q] = Cocc^T b Cvir, (ia|jb) = sum_Q B[i,a,Q] B[j,b,Q], then the pair sum of jues_rmp2.
 * The libint/psi4 integrals behind setup_df are not part of this library. */
JUES_API int jues_df_rmp2(jues_ctx *ctx, const double *pqP, int n, int naux, const double *Jpqh,
                          const double *Cocc, int o, const double *Cvir, int v, const double *eps,
                          int precision, double *e_out);

/* MP2 adjoint (no reference counterpart; the differentiation form): E as jues_rmp2 from the
 * full n x n MO matrix C (occupied columns first) and, scaled by e_bar,
 *   gao_bar[mu,nu,lam,sig] = dE/d(mu nu|lam sig)  (n^4, may be NULL)
 *   C_bar[mu,p]            = dE/dC[mu,p]          (n x n, may be NULL)
 * by back-transforming Gamma_iajb = 2(2K_iajb - K_ibja)/D.  The three-quarter transformed
 * integrals that C_bar needs are recomputed, not stored.  C_bar assumes 8-fold symmetric
 * AO integrals (real orbitals), as every ERI tensor has. */
JUES_API int jues_rmp2_adjoint(jues_ctx *ctx, const double *gao, int n, const double *C, int o,
                               const double *eps, int precision, double e_bar, double *e_out,
                               double *gao_bar, double *C_bar);

/* ---- batched MP2 (no reference counterpart; the batched form) --------------------------
 * Energies and, when the pointer arrays are given, adjoints of many independent closed-shell
 * systems of uneven size.  All systems run in one CUDA graph of grouped persistent launches (one
 * per stage, 12 stages with the adjoint); the graph is cached for a repeated batch signature.
 * precision: JUES_PREC_FP64 runs every stage as a grouped FP64 GETT; the split forms add, for
 * every stage whose contractions all have K <= 64 (all but the final dE/dC stage when every
 * nbf <= 64), the grouped three-plane tcgen05 GEMM as a candidate.  On first use each stage's
 * form is chosen by timing the candidates (autotuning).  Host arrays; gao_bar / C_bar are arrays
 * of nsys host pointers (entries may be NULL, the arrays themselves may be NULL). */
typedef struct {
    int n, o;             /* nbf and nocc; nvir = n - o                               */
    const double *gao;    /* n^4 AO integrals, column-major                            */
    const double *C;      /* n x n MO coefficients, occupied columns first             */
    const double *eps;    /* n orbital energies                                        */
} jues_mp2_system;

typedef struct {
    double upload_ms, graph_ms, download_ms;   /* CUDA-event times on the context stream */
    int graph_nodes;      /* kernels in the captured graph                              */
    int tuned;            /* 1 if this call built, autotuned and captured the plan       */
    int nstages;          /* grouped GETT stages                                         */
    int tile_shape[16];   /* chosen form per stage: FP64 tiles 0 64x64, 1 32x64, 2 64x32,
                             3 32x32; 4 the grouped three-plane tcgen05 GEMM             */
} jues_batch_info;

/* Which forms the batched entry point's autotuning may pick (no reference counterpart):
 * 0 = time every candidate (default), 1 = the FP64 tile shapes only, 2 = the grouped tcgen05
 * GEMM wherever it was built (split precision), FP64 tiles elsewhere. */
JUES_API int jues_ctx_set_batch_form(jues_ctx *ctx, int form);
JUES_API int jues_batch_rmp2(jues_ctx *ctx, int nsys, const jues_mp2_system *systems, int precision, double e_bar,
                             double *e_out, double **gao_bar, double **C_bar, jues_batch_info *info);

/* ---- coupled cluster ------------------------------------------------------------------
 * Whole solves.  t2_out (o*o*v*v, [i,j,a,b]) and t1_out (o*v, [i,a]) may be NULL; log may
 * be NULL, else it receives up to log_cap records.  Returns JUES_ENOTCONV (with e_out,
 * amplitudes and niter filled) when a convergence threshold was requested and not met. */
JUES_API int jues_cc_default_opts(jues_cc_opts *opts);
JUES_API int jues_rccd(jues_ctx *ctx, const double *gao, int n,
              const double *Cocc, int o, const double *Cvir, int v, const double *eps,
              const jues_cc_opts *opts, double *e_out, double *t2_out,
              jues_iter_log *log, int log_cap, int *niter);
JUES_API int jues_rccsd(jues_ctx *ctx, const double *gao, int n,
               const double *Cocc, int o, const double *Cvir, int v, const double *eps,
               const jues_cc_opts *opts, double *e_out, double *t1_out, double *t2_out,
               jues_iter_log *log, int log_cap, int *niter);

/* Fock matrix of a closed-shell determinant, IntegralTransformation.get_fock(wfn)
 * (src/Backend/IntegralTransformation.jl:119-141): f = C^T (h + 2J - K) C with the density of
 * the first nocc columns of C.  gao n^4, hao n x n, C n x nmo; f_out nmo x nmo; column-major. */
JUES_API int jues_get_fock(jues_ctx *ctx, const double *gao, const double *hao, int n, const double *C,
               int nmo, int nocc, double *f_out);

/* CCSD from a general (non-canonical) Fock matrix, AutoRCCSD.do_rccsd
 * (src/CoupledCluster/AutoRCCSD.jl:193-300): f = get_fock of C (the first ndocc columns
 * occupied), fcn frozen core orbitals, T1 = f_ov/d, T2 = <ij|ab>/D, iterations until
 * |dE| < opts.e_conv and max(||dT1||/len(T1), ||dT2||/len(T2)) < opts.r_conv, at most opts.maxit
 * (the reference's cc_max_iter = 50, cc_e_conv = cc_max_rms = 1e-10).  With do_pT the (T)
 * correction follows on the converged amplitudes with fo, fv = the Fock diagonal
 * (AutoRCCSD.jl:294-299).  Outputs may be NULL. */
JUES_API int jues_auto_rccsd(jues_ctx *ctx, const double *gao, const double *hao, int n, const double *C,
               int nmo, int ndocc, int fcn, const jues_cc_opts *opts, int do_pT, double *e_out,
               double *ept_out, double *t1_out, double *t2_out, jues_iter_log *log, int log_cap,
               int *niter);

/* (T) energy correction, PerturbativeTriples.compute_pT (src/CoupledCluster/
 * PerturbativeTriples.jl:35-138).  Host arrays, column-major, chemists' notation as the
 * reference takes them: T1[i,a] (o x v), T2[i,j,a,b] (o x o x v x v), Vvvvo[a,b,c,i] = (ab|ci)
 * (v x v x v x o), Vvooo[a,i,j,k] = (ai|jk) (v x o x o x o), Vvovo[a,i,b,j] = (ai|bj)
 * (v x o x v x o); fo (o) and fv (v) the Fock diagonals.  precision selects the arithmetic of
 * the W contractions (the energy sum is FP64). */
JUES_API int jues_pT(jues_ctx *ctx, const double *T1, const double *T2, const double *Vvvvo,
               const double *Vvooo, const double *Vvovo, const double *fo, const double *fv, int o,
               int v, int precision, double *e_out);
/* (T) on a CCSD session's current amplitudes and resident blocks, with fo, fv = eps
 * (AutoRCCSD.jl:294-299 with canonical orbitals). */
JUES_API int jues_cc_pT(jues_cc *cc, int precision, double *e_out);

/* Density-fitted CCD, DFRCCD.do_df_rccd (src/CoupledCluster/DF-RCCD.jl:11-54).  pqP[mu,nu,P]
 * and Jpqh as for jues_df_rmp2.  The four MO factors (DF-RCCD.jl:78-89) build the five blocks
 * once; the sweep is jues_rccd's.  The reference's own settings are guess = JUES_GUESS_MP2
 * (T2 = (ia|jb)/D, DF-RCCD.jl:119-137), diis = 0, r_conv = 0, maxit = 40.  variant selects
 * DF-RCCD.jl's WmBeJ (JUES_DF_REFERENCE) or RCCD.jl's (JUES_DF_RCCD). */
JUES_API int jues_df_rccd(jues_ctx *ctx, const double *pqP, int n, int naux, const double *Jpqh,
               const double *Cocc, int o, const double *Cvir, int v, const double *eps,
               const jues_cc_opts *opts, int variant, double *e_out, double *t2_out,
               jues_iter_log *log, int log_cap, int *niter);

/* Resident CC sessions: integrals and amplitudes stay in device memory between calls, so
 * a caller can time single sweeps.  method: 0 = CCD, 1 = CCSD.  gao_is_device != 0 means
 * gao is a device pointer on the context's device. */
JUES_API int jues_cc_create(jues_ctx *ctx, int method, const double *gao, int gao_is_device, int n,
                   const double *Cocc, int o, const double *Cvir, int v, const double *eps,
                   const jues_cc_opts *opts, jues_cc **out);
/* The same session for CCD on density-fitted integrals (DF-RCCD.jl:11-54): pqP and Jpqh as for
 * jues_df_rmp2 (pqP_is_device != 0: pqP is a device pointer), variant JUES_DF_*. */
JUES_API int jues_cc_create_df(jues_ctx *ctx, const double *pqP, int pqP_is_device, int n, int naux,
                   const double *Jpqh, const double *Cocc, int o, const double *Cvir, int v,
                   const double *eps, const jues_cc_opts *opts, int variant, jues_cc **out);
/* Run up to nsweeps sweeps (stopping early on convergence); *done = sweeps run,
 * *converged = 1 if the thresholds were met. */
JUES_API int jues_cc_iterate(jues_cc *cc, int nsweeps, int *done, int *converged);
JUES_API int jues_cc_set_precision(jues_cc *cc, int precision);
JUES_API int jues_cc_energy(jues_cc *cc, double *e_out);
JUES_API int jues_cc_amplitudes(jues_cc *cc, double *t1_out, double *t2_out);
JUES_API int jues_cc_log(jues_cc *cc, jues_iter_log *log, int log_cap, int *count);
JUES_API int jues_cc_destroy(jues_cc *cc);

#ifdef __cplusplus
}
#endif
#endif /* JUES_GPU_H */
