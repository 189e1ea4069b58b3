// Split-precision (BF16 hi+lo, three products, FP32 accumulation) GEMM on the tcgen05 tensor
// cores.  Placeholder until the tcgen05 kernel lands: refuses loudly.
#include "common.cuh"

namespace jues {

struct PackCache {};

void gett_tc(Ctx *, const GettArgs &, const char *) {
    throw Error(JUES_EINVAL, "split-BF16 precision is not available in this build");
}
void pack_cache_clear(Ctx *) {}
void pack_cache_destroy(PackCache *p) { delete p; }
void pack_cache_drop(Ctx *, const void *) {}

}  // namespace jues
