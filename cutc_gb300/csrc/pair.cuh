// Pair-term (grad1 u) kernels: argument block and launchers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cutc {

// (f, d f/dx, d f/dy, d f/dz) of one (point, nucleus) pair
struct __align__(32) NucTerm {
    double f, gx, gy, gz;
};

struct PairArgs {
    int i0;            // first r1 row of the tile (global index)
    int n1b;           // r1 rows in the tile
    int n2;            // r2 points
    int nN;            // nuclei
    int n_terms;       // Jastrow terms kept (|c| >= 1e-10)
    const double *r1;  // (3, n_grid1) AoS
    const double *r2;  // (3, n2) AoS
    const NucTerm *t1; // [n1b][nN] (f1, grad f1) of the tile's rows
    const double *f2;  // [nN][n2]
    const double *coef;     // [n_terms][3] = (c m, c n, c o)
    const int *exps;        // [n_terms] = m | n << 3 | o << 6
    const int *term_off;    // [nN + 1] first term of each nucleus
    double a_ee;
    double *G;         // G[c * plane + i * ldg + j]
    int64_t ldg;
    int64_t plane;
};

int launch_r1_terms(cudaStream_t st, int i0, int n, int nN, const double *r1, const double *rn,
                    double a, NucTerm *t1);
int launch_r2_terms(cudaStream_t st, int n2, int nN, const double *r2, const double *rn,
                    double a, double *f2);
int launch_pair_f64(cudaStream_t st, const PairArgs &P);

}  // namespace cutc
