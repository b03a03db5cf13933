// AO values and gradients from a Cartesian Gaussian basis (device).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cutc_int.h"
#include "engine.cuh"

namespace cutc {

constexpr int kMaxAoPower = 8;  // Cartesian power per axis
constexpr int kMaxPrim = 64;    // primitives per function

// The basis in device memory (one upload of a few KB per build).
struct BasisDev {
    int n_ao = 0;
    const double *center = nullptr;  // (n_ao, 3)
    const double *exp = nullptr, *coef = nullptr;
    const int *power = nullptr;      // (n_ao, 3)
    const int *offset = nullptr;     // (n_ao + 1)
};

int validate_basis(const cutc_basis *b, int n_ao);
int upload_basis(Workspace &W, int slot, cudaStream_t st, const cutc_basis *b, BasisDev *out);
// out[(c * n_ao + a) * ld + g], c < comps (1: value; 4: value and gradient), r (n, 3) AoS
int launch_eval_aos(cudaStream_t st, const BasisDev &B, int n, const double *r, int comps,
                    double *out, int64_t ld);

}  // namespace cutc
