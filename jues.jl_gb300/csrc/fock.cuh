#pragma once
#include "common.cuh"

namespace jues {

// f (nmo x nmo) = C^T (h + 2 J[D] - K[D]) C with D = Co Co^T (src/Backend/IntegralTransformation.jl:
// 119-141).  g: n^4 AO integrals, h: n x n core Hamiltonian, C: n x nmo, Co: n x o; all device,
// column-major.
void get_fock(Ctx *ctx, const double *g, const double *h, int n, const double *C, int nmo, const double *Co, int o,
              double *f);

}  // namespace jues
