// Index-order helpers of the two-electron arrays, under the reference's names.
//
// The reference ships them for its cutc_no path (src/add_trans_inplace.cu,
// src/trans_pqst_psqt_inplace.cu, src/trans_pqst_psqt_copy.cu): one thread per
// (p, t) walks all (q, s) with strided, uncoalesced accesses.  Here every
// access is coalesced: the symmetrisation works on 32 x 32 tile pairs staged in
// shared memory, and the (q, s) swap moves whole p-vectors (the fastest index)
// with consecutive threads on consecutive p.  Same signatures, device
// pointers, legacy default stream and no host synchronisation, as the reference.
#include <cuda_runtime.h>

#include "common.cuh"
#include "products.cuh"

namespace cutc {

// a <- a + a^T, column-major n x n; block (bi, bj), bj <= bi, owns the tile pair
// (bi, bj) / (bj, bi), read completely before either is written.
__global__ void add_transpose_kernel(double *__restrict__ a, int n)
{
    const int bi = blockIdx.x, bj = blockIdx.y;
    if (bj > bi)
        return;
    __shared__ double t1[32][33], t2[32][33];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = bi * 32, j0 = bj * 32;
    // t1[c][r] = a(i0 + r, j0 + c), t2[c][r] = a(j0 + r, i0 + c)
    for (int c = ty; c < 32; c += blockDim.y) {
        const int r = tx;
        t1[c][r] = (i0 + r < n && j0 + c < n) ? a[(i0 + r) + (int64_t)n * (j0 + c)] : 0.0;
        t2[c][r] = (j0 + r < n && i0 + c < n) ? a[(j0 + r) + (int64_t)n * (i0 + c)] : 0.0;
    }
    __syncthreads();
    for (int c = ty; c < 32; c += blockDim.y) {
        const int r = tx;
        // a(i0 + r, j0 + c) += a(j0 + c, i0 + r) = t2[r][c]
        if (i0 + r < n && j0 + c < n)
            a[(i0 + r) + (int64_t)n * (j0 + c)] = t1[c][r] + t2[r][c];
        if (bi != bj && j0 + r < n && i0 + c < n)
            a[(j0 + r) + (int64_t)n * (i0 + c)] = t2[c][r] + t1[r][c];
    }
}

// data(p, q, s, t) <-> data(p, s, q, t) for q < s: block (s, t) swaps the p-vectors
// of every q < s (disjoint pairs, so blocks never touch the same element).
__global__ void swap_qs_kernel(double *__restrict__ d, int n)
{
    const int s = blockIdx.x, t = blockIdx.y;
    const int64_t n2 = (int64_t)n * n, base = (int64_t)t * n2 * n;
    for (int q = 0; q < s; q++) {
        double *x = d + base + (int64_t)q * n + (int64_t)s * n2;
        double *y = d + base + (int64_t)s * n + (int64_t)q * n2;
        for (int p = threadIdx.x; p < n; p += blockDim.x) {
            const double v = x[p];
            x[p] = y[p];
            y[p] = v;
        }
    }
}

// dst(p, q, s, t) = src(p, s, q, t): block (s, t) writes the p-vectors of all q
__global__ void copy_qs_kernel(const double *__restrict__ src, double *__restrict__ dst, int n)
{
    const int s = blockIdx.x, t = blockIdx.y;
    const int64_t n2 = (int64_t)n * n, base = (int64_t)t * n2 * n;
    for (int q = 0; q < n; q++) {
        double *x = dst + base + (int64_t)q * n + (int64_t)s * n2;
        const double *y = src + base + (int64_t)s * n + (int64_t)q * n2;
        for (int p = threadIdx.x; p < n; p += blockDim.x)
            x[p] = y[p];
    }
}

static bool check_launch(const char *what, int size)
{
    if (size < 0 || size > 65535) {
        cutc_set_error(CUTC_ERR_INVALID, "%s: size %d outside [0, 65535]", what, size);
        return false;
    }
    return true;
}

static void record(const char *what)
{
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        cutc_set_error(CUTC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int launch_add_transpose(cudaStream_t st, double *a, int n)
{
    const unsigned nb = ceil_div(n, 32);
    if (n <= 0)
        return CUTC_OK;
    if (nb > 65535u) {
        cutc_set_error(CUTC_ERR_INVALID, "A + A^T of order %d: too large", n);
        return CUTC_ERR_INVALID;
    }
    add_transpose_kernel<<<dim3(nb, nb), dim3(32, 8), 0, st>>>(a, n);
    CUTC_CUDA_TRY(cudaGetLastError());
    note_launches(1);
    return CUTC_OK;
}

int launch_swap_qs(cudaStream_t st, double *d, int n)
{
    if (n <= 0)
        return CUTC_OK;
    if (n > 65535) {
        cutc_set_error(CUTC_ERR_INVALID, "(q, s) swap of order %d: too large", n);
        return CUTC_ERR_INVALID;
    }
    swap_qs_kernel<<<dim3(n, n), 128, 0, st>>>(d, n);
    CUTC_CUDA_TRY(cudaGetLastError());
    note_launches(1);
    return CUTC_OK;
}

}  // namespace cutc

using namespace cutc;

extern "C" void trans_inplace(double *data, int size)
{
    if (size <= 0 || !data)
        return;
    const unsigned nb = ceil_div(size, 32);
    if (nb > 65535u) {
        cutc_set_error(CUTC_ERR_INVALID, "trans_inplace: size %d too large", size);
        return;
    }
    add_transpose_kernel<<<dim3(nb, nb), dim3(32, 8)>>>(data, size);
    note_launches(1);
    record("trans_inplace");
}

extern "C" void trans_pqst_psqt_inplace(int size, double *data)
{
    if (size <= 0 || !data || !check_launch("trans_pqst_psqt_inplace", size))
        return;
    swap_qs_kernel<<<dim3(size, size), 128>>>(data, size);
    note_launches(1);
    record("trans_pqst_psqt_inplace");
}

extern "C" void trans_pqst_psqt_copy(int size, double *data_old, double *data_new)
{
    if (size <= 0 || !data_old || !data_new || !check_launch("trans_pqst_psqt_copy", size))
        return;
    copy_qs_kernel<<<dim3(size, size), 128>>>(data_old, data_new, size);
    note_launches(1);
    record("trans_pqst_psqt_copy");
}
