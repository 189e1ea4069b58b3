#pragma once
#include <string>
#include <utility>
#include <vector>

#include "common.cuh"

namespace jues {
// flops of the cost-ordered four quarter transforms
double transform4_flops(int n, const int d[4]);
// device pointers; a null C[p] leaves index p in the AO basis; out element (x0,x1,x2,x3) of the chemists' block goes to sum_q x_q*ostr[q]
// din: the input's extents when it is not n^4 (indices with a null C keep theirs)
void transform4(Ctx *ctx, int prec, const double *g, int n, const double *const C[4], const int d[4],
                double *out, const long long ostr[4], bool g_const, const long long *din = nullptr);
// out[mu,nu,lam,sig] = sum X[i,a,j,b] C1[mu,i] C2[nu,a] C3[lam,j] C4[sig,b], out n^4 column-major
void backtransform4(Ctx *ctx, int prec, const double *X, const int d[4], int n, const double *const C[4],
                    double *out);
// the GETT steps of transform4 / backtransform4 with caller-provided ping-pong buffers of
// transform4_scratch / backtransform4_scratch elements each (used by the batched form)
std::vector<GettArgs> transform4_plan(const double *g, int n, const double *const C[4], const int d[4],
                                      double *out, const long long ostr[4], double *buf0, double *buf1,
                                      const long long *din = nullptr);
long long transform4_scratch(int n, const double *const C[4], const int d[4], const long long *din = nullptr);
std::vector<GettArgs> backtransform4_plan(const double *X, const int d[4], int n, const double *const C[4],
                                          double *out, double *buf0, double *buf1);
long long backtransform4_scratch(const int d[4], int n);
// spec: 4 chars of o/O/v/V; phys: physicists' notation; fcn: frozen core count
void get_eri_block(Ctx *ctx, int prec, const double *g, int n, const double *Cocc, int o,
                   const double *Cvir, int v, const char spec[4], bool phys, int fcn, double *out,
                   bool g_const);
// several blocks of one integral array: blocks whose first quarter steps coincide (same index
// contracted with the same coefficients) share them (the occupied blocks' first quarter)
void get_eri_blocks(Ctx *ctx, int prec, const double *g, int n, const double *Cocc, int o, const double *Cvir,
                    int v, const std::vector<std::pair<std::string, double *>> &blocks, bool phys, int fcn,
                    bool g_const);
}  // namespace jues
