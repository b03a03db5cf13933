// Split-precision (BF16-slice) contractions: plan and entry points.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.cuh"

namespace cutc {

constexpr int kMaxSlices = 7;
constexpr int kDefaultSlices = 5;

struct SplitPlan {
    int slot0 = 0;
    int n_slices = 0;
    int64_t n1t = 0;
    void *a_slices = nullptr;  // P slices (X-build A operand)
    float *a_scale = nullptr;
    void *b_slices = nullptr;  // G-tile slices (X-build B operand)
    float *b_scale = nullptr;
};

size_t split_r1_row_bytes(const Request &R);
int split_prepare_x(Engine *E, const Request &R, cudaStream_t st, const double *wr2,
                    const double *aos2v, int64_t n1t, int slot0, SplitPlan &sp);
int split_x_tile(Engine *E, const Request &R, cudaStream_t st, SplitPlan &sp, const double *G,
                 int i0, int nb, double *Xp);
int split_int2e(Engine *E, const Request &R, cudaStream_t st, SplitPlan &sp, const double *wr1,
                const double *aos1, const double *Xp, double *I);

}  // namespace cutc
