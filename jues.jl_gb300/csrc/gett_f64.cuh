#pragma once
#include <vector>

#include "common.cuh"

namespace jues {

// one GETT of a grouped launch (device-resident descriptor)
struct GroupProblem {
    long long M, N, K;
    double alpha, beta;
    const double *A; Mode mA, kA;
    const double *B; Mode kB, nB;
    double *C; Mode mC, nC;
    const double *Cin;
    long long mtiles;       // row tiles for the chosen tile shape
    long long tile_start;   // first global tile of this problem
};

struct TileShape {
    int bm, bn;
};
constexpr int kNumTileShapes = 4;
extern const TileShape kTileShapes[kNumTileShapes];

GroupProblem to_problem(const GettArgs &a);
// fills mtiles / tile_start for the shape; returns the total tile count
long long grouped_tiles(std::vector<GroupProblem> &probs, int shape);
// persistent grouped FP64 GETT over device descriptors
void gett_f64_grouped_launch(Ctx *ctx, const GroupProblem *d_probs, int nprob, long long total, int shape,
                             const char *name);

}  // namespace jues
