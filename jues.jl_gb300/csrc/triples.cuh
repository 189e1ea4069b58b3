#pragma once
#include "common.cuh"

namespace jues {

// A four-index array read through element strides: x[i0,i1,i2,i3] = p[i0 s0 + i1 s1 + i2 s2 + i3 s3].
// The (T) inputs arrive either as the reference's chemists'-notation arrays (column-major) or
// as views of the CCSD blocks, which are the same numbers in another index order.
struct View4 {
    const double *p = nullptr;
    long long s[4] = {0, 0, 0, 0};
};
inline View4 col_major(const double *p, long long d0, long long d1, long long d2) {
    View4 v;
    v.p = p;
    v.s[0] = 1; v.s[1] = d0; v.s[2] = d0 * d1; v.s[3] = d0 * d1 * d2;
    return v;
}

// (T) energy correction, compute_pT (src/CoupledCluster/PerturbativeTriples.jl:35-138).
// T1[i,a] (o x v) and T2[i,j,a,b] (o x o x v x v) column-major on the device;
// Vvvvo[a,b,c,i] = (ab|ci), Vvooo[a,i,j,k] = (ai|jk), Vvovo[a,i,b,j] = (ai|bj); fo, fv the Fock
// diagonals (device).  prec selects the arithmetic of the W contractions.
double pT_energy(Ctx *ctx, int prec, const double *T1, const double *T2, const View4 &Vvvvo, const View4 &Vvooo,
                 const View4 &Vvovo, const double *fo, const double *fv, int o, int v);

double pT_flops(int o, int v);   // 2 o^3 v^3 (v + o) summed over i >= j >= k, as executed

}  // namespace jues
