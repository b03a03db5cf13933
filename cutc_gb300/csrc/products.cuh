// Pair-product, expansion and assembly kernels: launchers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cutc {

// out[tri(a,b) * ld + g] = w[g] chi_a(g) chi_b(g); chi[a * ld_chi + g]
int launch_sym_products(cudaStream_t st, int n, int nA, const double *w, const double *chi,
                        int64_t ld_chi, double *out, int64_t ld);
// out[stri(c,d) * ld + m n + g] = w (chi_c d_m chi_d - chi_d d_m chi_c), c > d;
// aos[(k nA + a) ld_aos + g] is component k of AO a at grid point g
int launch_antisym_products(cudaStream_t st, int n, int nA, const double *w, const double *aos,
                            int64_t ld_aos, double *out, int64_t ld);
// full AO-pair rows from packed rows
int launch_expand_pairs(cudaStream_t st, int64_t rows, int nA, const double *Xp, int64_t ldp,
                        double *X);
// Columns c0 <= col < c1 of int_2e = A + A^T (column-major, nA^2 rows) from the
// packed symmetric (H) and antisymmetric (N) parts; out holds column c0 first.
// psqt: element (p,q,s,t) goes where (p,s,q,t) would (c0 and c1 multiples of nA).
int launch_assemble_int2e(cudaStream_t st, int nA, const double *H, const double *N, int c0,
                          int c1, bool psqt, double *out);
// a <- a + a^T (column-major n x n), and the (p,q,s,t) -> (p,s,q,t) swap of an n^4 array,
// on a stream (layout.cu; the reference-named helpers use the legacy default stream)
int launch_add_transpose(cudaStream_t st, double *a, int n);
int launch_swap_qs(cudaStream_t st, double *d, int n);

}  // namespace cutc
