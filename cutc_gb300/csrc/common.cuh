// Shared definitions of the GB300 transcorrelated-integral engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <atomic>

#include "cutc_int.h"

#define CUTC_CUDA_TRY(expr)                                                   \
    do {                                                                      \
        cudaError_t cutc_err_ = (expr);                                       \
        if (cutc_err_ != cudaSuccess) {                                       \
            cutc_set_error(CUTC_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, \
                           #expr, cudaGetErrorString(cutc_err_));             \
            return cutc_err_ == cudaErrorMemoryAllocation ? CUTC_ERR_NO_MEMORY \
                                                          : CUTC_ERR_CUDA;    \
        }                                                                     \
    } while (0)

// (the status variable has a name no caller uses, so that expr may name any
// variable of the caller)
#define CUTC_TRY(expr)                    \
    do {                                  \
        int cutc_status_ = (expr);        \
        if (cutc_status_ != CUTC_OK)      \
            return cutc_status_;          \
    } while (0)

// Records the message behind the last non-zero status (thread-local).
void cutc_set_error(int status, const char *fmt, ...);

namespace cutc {

// Jastrow exponents are evaluated by repeated multiplication up to this power
// (src/jast_bh.cu:3-28 leaves larger exponents undefined; we reject them).
constexpr int kMaxExp = 6;
// Largest nucleus count / term count per nucleus the kernels stage in shared
// memory.  Larger inputs are rejected with CUTC_ERR_INVALID.
constexpr int kMaxNuc = 128;
constexpr int kMaxTerms = 4096;

// Packed index of the pair (a, b), a >= b, in the lower triangle stored
// column by column: consecutive a give consecutive indices, and so do the
// full indices a + nA b, which keeps gathers and scatters coalesced.
__host__ __device__ inline int64_t tri_index(int a, int b, int n)
{
    return (int64_t)b * (2 * n - b + 1) / 2 + (a - b);
}

// Packed index of the strict lower triangle (a > b).
__host__ __device__ inline int64_t stri_index(int a, int b, int n)
{
    return (int64_t)b * (2 * n - b - 1) / 2 + (a - b - 1);
}

inline int64_t n_pairs(int n) { return (int64_t)n * (n + 1) / 2; }
inline int64_t n_strict_pairs(int n) { return (int64_t)n * (n - 1) / 2; }

inline unsigned ceil_div(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

// Counts kernel launches of this library (reported in cutc_stats).
void note_launches(int n);

// The bit of the current device in a per-device "done" mask.  Function
// attributes (the dynamic shared-memory opt-in) are set per device, so a flag
// kept for the whole process would skip a second device.
inline unsigned long long current_device_bit()
{
    int dev = 0;
    cudaGetDevice(&dev);
    return 1ull << (dev & 63);
}

}  // namespace cutc
