#pragma once
#include "common.cuh"

namespace jues {
// flops of the cost-ordered four quarter transforms
double transform4_flops(int n, const int d[4]);
// device pointers; out element (x0,x1,x2,x3) of the chemists' block goes to sum_q x_q*ostr[q]
void transform4(Ctx *ctx, int prec, const double *g, int n, const double *const C[4], const int d[4],
                double *out, const long long ostr[4], bool g_const);
// spec: 4 chars of o/O/v/V; phys: physicists' notation; fcn: frozen core count
void get_eri_block(Ctx *ctx, int prec, const double *g, int n, const double *Cocc, int o,
                   const double *Cvir, int v, const char spec[4], bool phys, int fcn, double *out,
                   bool g_const);
}  // namespace jues
