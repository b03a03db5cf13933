// Grid pair products, X expansion and int_2e assembly (sm_103a).
//
// The reference materialises the full nA^2 pair products
//   P[j + nA i][r2]  = w2 chi_i chi_j                       (src/long_range_integ.cu:39)
//   S0[j + nA i][r1] = w1 chi_i chi_j                       (src/short_range_integ_herm.cu:38)
//   S[j + nA i][m][r1] = w1 (chi_j d_m chi_i - chi_i d_m chi_j)   (src/short_range_integ_nonherm.cu:55)
// with one thread per grid point writing nA^2 values at stride n.  Here:
//   * P and S0 are symmetric in the AO pair, so only the lower triangle
//     (a >= b, tri_index) is built: half the memory and half the GEMM work;
//   * S is antisymmetric, so only the strict lower triangle is built;
//   * threads run along the grid index, so every store is coalesced.
// The symmetric/antisymmetric halves are recombined in assemble_int2e_kernel,
// which also performs the reference's A + A^T (src/add_trans_inplace.cu:2-21)
// without materialising A.
#include "common.cuh"
#include "products.cuh"

namespace cutc {

// out[tri(a, b) * ld + g] = w[g] chi_a(g) chi_b(g), b <= a, g in [0, n)
__global__ void sym_products_kernel(int n, int nA, const double *__restrict__ w,
                                    const double *__restrict__ chi, int64_t ld_chi,
                                    double *__restrict__ out, int64_t ld)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int a = blockIdx.y;
    if (g >= n)
        return;
    const double wa = w[g] * chi[(int64_t)a * ld_chi + g];
    for (int b = 0; b <= a; b++)
        out[tri_index(a, b, nA) * ld + g] = wa * chi[(int64_t)b * ld_chi + g];
}

// out[stri(c, d) * ld + m * n + g] = w (chi_c d_m chi_d - chi_d d_m chi_c), c > d
// aos is the (ld_aos, nA, 4) array seen from the first of the n grid points;
// component k of AO a at aos[(k * nA + a) * ld_aos + g].
__global__ void antisym_products_kernel(int n, int nA, const double *__restrict__ w,
                                        const double *__restrict__ aos, int64_t ld_aos,
                                        double *__restrict__ out, int64_t ld)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (g >= n)
        return;
    const int64_t comp = (int64_t)nA * ld_aos;
    const double wg = w[g];
    const double vc = aos[(int64_t)c * ld_aos + g];
    const double dc0 = aos[comp + (int64_t)c * ld_aos + g];
    const double dc1 = aos[2 * comp + (int64_t)c * ld_aos + g];
    const double dc2 = aos[3 * comp + (int64_t)c * ld_aos + g];
    for (int d = 0; d < c; d++) {
        const double vd = aos[(int64_t)d * ld_aos + g];
        double *o = out + stri_index(c, d, nA) * ld + g;
        o[0] = wg * (vc * aos[comp + (int64_t)d * ld_aos + g] - vd * dc0);
        o[n] = wg * (vc * aos[2 * comp + (int64_t)d * ld_aos + g] - vd * dc1);
        o[2 * (int64_t)n] = wg * (vc * aos[3 * comp + (int64_t)d * ld_aos + g] - vd * dc2);
    }
}

// X[(row) * nA^2 + a + nA b] = Xp[(row) * ldp + tri(max(a,b), min(a,b))] for
// rows = m * n1 + i of the requested components.
__global__ void expand_pairs_kernel(int64_t rows, int nA, const double *__restrict__ Xp, int64_t ldp,
                                    double *__restrict__ X)
{
    const int64_t nA2 = (int64_t)nA * nA;
    const int64_t row = blockIdx.y + (int64_t)gridDim.y * blockIdx.z;
    if (row >= rows)
        return;
    const double *src = Xp + row * ldp;
    double *dst = X + row * nA2;
    // nA^2 < 2^30 (the build's argument checks): 32-bit index arithmetic, one division
    const int n2 = (int)nA2;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n2; k += gridDim.x * blockDim.x) {
        const int b = k / nA, a = k - b * nA;
        dst[k] = src[a >= b ? tri_index(a, b, nA) : tri_index(b, a, nA)];
    }
}

// A[(a,b), (c,d)] from the packed contractions:
//   H[p + np q]  symmetric part  (p = tri(a,b), q = tri(c,d))
//   N[p + np l]  antisymmetric part, l = stri(max(c,d), min(c,d)), sign + if c > d
__device__ __forceinline__ double a_entry(int row, int col, int nA, int64_t np,
                                          const double *__restrict__ H,
                                          const double *__restrict__ N)
{
    const int a = row % nA, b = row / nA, c = col % nA, d = col / nA;
    const int64_t p = a >= b ? tri_index(a, b, nA) : tri_index(b, a, nA);
    const int64_t q = c >= d ? tri_index(c, d, nA) : tri_index(d, c, nA);
    double v = H[p + np * q];
    if (c > d)
        v += N[p + np * stri_index(c, d, nA)];
    else if (c < d)
        v -= N[p + np * stri_index(d, c, nA)];
    return v;
}

// out[row + n (col - c0)] = A[row, col] + A[col, row] for the columns
// c0 <= col < c1, n = nA^2, 32x32 tiles.  PSQT: row = p + nA q, col = s + nA t
// goes to p + nA s + nA^2 q + nA^3 (t - c0 / nA) instead.
template <bool PSQT>
__global__ void assemble_int2e_kernel(int nA, const double *__restrict__ H,
                                      const double *__restrict__ N, int c0, int c1,
                                      double *__restrict__ out)
{
    __shared__ double t[32][33];
    const int n = nA * nA;
    const int64_t np = (int64_t)nA * (nA + 1) / 2;
    const int R0 = blockIdx.x * 32, C0 = c0 + blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    double v[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int row = R0 + tx, col = C0 + ty + 8 * k;
        v[k] = (row < n && col < c1) ? a_entry(row, col, nA, np, H, N) : 0.0;
        // transposed term, computed with tx running along A's row index
        const int row2 = C0 + tx, col2 = R0 + ty + 8 * k;
        t[ty + 8 * k][tx] = (row2 < c1 && col2 < n) ? a_entry(row2, col2, nA, np, H, N) : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int row = R0 + tx, col = C0 + ty + 8 * k;
        // t[i][j] = A[C0 + j, R0 + i]  ->  A[col, row] = t[tx][ty + 8k]
        if (row < n && col < c1) {
            int64_t o;
            if (PSQT) {
                const int p = row % nA, q = row / nA, s_ = col % nA, tt = col / nA - c0 / nA;
                o = p + (int64_t)nA * s_ + (int64_t)n * q + (int64_t)n * nA * tt;
            } else {
                o = row + (int64_t)n * (col - c0);
            }
            out[o] = v[k] + t[tx][ty + 8 * k];
        }
    }
}

int launch_sym_products(cudaStream_t st, int n, int nA, const double *w, const double *chi,
                        int64_t ld_chi, double *out, int64_t ld)
{
    if (n <= 0)
        return CUTC_OK;
    dim3 grid(ceil_div(n, 128), nA);
    sym_products_kernel<<<grid, 128, 0, st>>>(n, nA, w, chi, ld_chi, out, ld);
    CUTC_CUDA_TRY(cudaGetLastError());
    return CUTC_OK;
}

int launch_antisym_products(cudaStream_t st, int n, int nA, const double *w, const double *aos,
                            int64_t ld_aos, double *out, int64_t ld)
{
    if (n <= 0 || nA < 2)
        return CUTC_OK;
    dim3 grid(ceil_div(n, 128), nA);
    antisym_products_kernel<<<grid, 128, 0, st>>>(n, nA, w, aos, ld_aos, out, ld);
    CUTC_CUDA_TRY(cudaGetLastError());
    return CUTC_OK;
}

int launch_expand_pairs(cudaStream_t st, int64_t rows, int nA, const double *Xp, int64_t ldp,
                        double *X)
{
    if (rows <= 0)
        return CUTC_OK;
    const int64_t nA2 = (int64_t)nA * nA;
    unsigned gx = ceil_div(nA2, 256);
    if (gx > 64)
        gx = 64;
    unsigned gy = rows < 65535 ? (unsigned)rows : 65535u;
    unsigned gz = ceil_div(rows, gy);
    expand_pairs_kernel<<<dim3(gx, gy, gz), 256, 0, st>>>(rows, nA, Xp, ldp, X);
    CUTC_CUDA_TRY(cudaGetLastError());
    return CUTC_OK;
}

int launch_assemble_int2e(cudaStream_t st, int nA, const double *H, const double *N, int c0,
                          int c1, bool psqt, double *out)
{
    const int n = nA * nA;
    if (c0 < 0 || c1 > n || c0 >= c1)
        return CUTC_OK;
    if (psqt && (c0 % nA || c1 % nA)) {
        cutc_set_error(CUTC_ERR_INVALID, "int_2e slab [%d, %d) is not a whole number of t", c0, c1);
        return CUTC_ERR_INVALID;
    }
    dim3 grid(ceil_div(n, 32), ceil_div(c1 - c0, 32));
    if (psqt)
        assemble_int2e_kernel<true><<<grid, dim3(32, 8), 0, st>>>(nA, H, N, c0, c1, out);
    else
        assemble_int2e_kernel<false><<<grid, dim3(32, 8), 0, st>>>(nA, H, N, c0, c1, out);
    CUTC_CUDA_TRY(cudaGetLastError());
    return CUTC_OK;
}

}  // namespace cutc
