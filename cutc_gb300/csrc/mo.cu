// X in the molecular-orbital basis, in the order the reference's cutc_no reads it.
//
// cutc_int returns X in the AO basis as X_ao(a, b, g, m) (src/cutc_module.f90:34,
// column-major, AO pair fastest); cutc_no reads the MO-basis X as
// X_mo(g, m, i, j) with the grid point fastest (src/no_tmpJ_cs_kernel.cu:18-30,
// index g + n1 m + 3 n1 i + 3 n1 n_mo j).  The transform between them is done by
// the caller in the reference's workflow; here it is
//     X_mo(g, m, i, j) = sum_{a, b} L(a, i) X_ao(a, b, g, m) R(b, j)
// with L and R the left and right MO coefficients (n_ao x n_mo, column-major;
// L = R for a symmetric orbital set), per r1 block and component:
//     T(i, b, g) = sum_a L(a, i) X(a, b, g)        one DGEMM (n_mo x n_ao*nb x n_ao)
//     Y(i, j, g) = sum_b T(i, b, g) R(b, j)        strided-batched DGEMM over g
//     X_mo(g, m, i, j) = Y(i, j, g)               tiled transpose (coalesced both ways)
// FP64 throughout (the FP64 DMMA GEMM of the plain form), which is 4 n_mo n_ao (n_ao + n_mo) n1 flops
// per component.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "dgemm.cuh"
#include "engine.cuh"

namespace cutc {

// dst[r + ldd * c] = src[c + lds * r] for r < rows, c < cols (32 x 32 tiles)
__global__ void transpose_kernel(const double *__restrict__ src, int64_t lds, int rows, int cols,
                                 double *__restrict__ dst, int64_t ldd)
{
    __shared__ double t[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int r = r0 + k, c = c0 + threadIdx.x;
        t[k][threadIdx.x] = (r < rows && c < cols) ? src[c + lds * r] : 0.0;
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int c = c0 + k, r = r0 + threadIdx.x;
        if (r < rows && c < cols)
            dst[r + ldd * c] = t[threadIdx.x][k];
    }
}

static int launch_transpose(cudaStream_t st, const double *src, int64_t lds, int rows, int cols,
                            double *dst, int64_t ldd)
{
    if (rows <= 0 || cols <= 0)
        return CUTC_OK;
    if (ceil_div(rows, 32) > 65535u) {
        cutc_set_error(CUTC_ERR_INVALID, "transpose of %d rows exceeds the grid", rows);
        return CUTC_ERR_INVALID;
    }
    dim3 grid(ceil_div(cols, 32), ceil_div(rows, 32));
    transpose_kernel<<<grid, dim3(32, 8), 0, st>>>(src, lds, rows, cols, dst, ldd);
    CUTC_CUDA_TRY(cudaGetLastError());
    note_launches(1);
    return CUTC_OK;
}

enum MoSlot { M_L = 180, M_R, M_T, M_Y, M_XIN, M_XOUT };

static int x_ao_to_mo(Engine *E, cudaStream_t st, int n1, int nA, int n_mo, int comps,
                      const double *L, const double *R, const double *x_ao, double *x_mo,
                      bool dev, size_t budget)
{
    Workspace &W = E->ws;
    void *p;
    const double *dL = L, *dR = R;
    const size_t cbytes = (size_t)nA * n_mo * 8;
    if (!dev) {
        CUTC_TRY(W.get(M_L, cbytes, &p));
        CUTC_CUDA_TRY(cudaMemcpyAsync(p, L, cbytes, cudaMemcpyHostToDevice, st));
        dL = (const double *)p;
        CUTC_TRY(W.get(M_R, cbytes, &p));
        CUTC_CUDA_TRY(cudaMemcpyAsync(p, R, cbytes, cudaMemcpyHostToDevice, st));
        dR = (const double *)p;
    }
    // r1 points per block: T, Y (and the host-mode staging of X_ao and X_mo)
    const size_t per_g = ((size_t)n_mo * nA + (size_t)n_mo * n_mo +
                          (dev ? 0 : (size_t)nA * nA + (size_t)n_mo * n_mo)) * 8;
    int nb = (int)std::max<size_t>(1, std::min<size_t>((size_t)n1, budget / per_g));
    double *T, *Y, *Xin = nullptr, *Xout = nullptr;
    CUTC_TRY(W.get(M_T, (size_t)n_mo * nA * nb * 8, &p));
    T = (double *)p;
    CUTC_TRY(W.get(M_Y, (size_t)n_mo * n_mo * nb * 8, &p));
    Y = (double *)p;
    if (!dev) {
        CUTC_TRY(W.get(M_XIN, (size_t)nA * nA * nb * 8, &p));
        Xin = (double *)p;
        CUTC_TRY(W.get(M_XOUT, (size_t)n_mo * n_mo * nb * 8, &p));
        Xout = (double *)p;
    }
    const double one = 1.0, zero = 0.0;
    const int64_t nA2 = (int64_t)nA * nA, nm2 = (int64_t)n_mo * n_mo;
    const int64_t ldo = (int64_t)comps * n1;  // X_mo: g + n1 m + ldo (i + n_mo j)
    for (int m = 0; m < comps; m++) {
        for (int g0 = 0; g0 < n1; g0 += nb) {
            const int gb = std::min(nb, n1 - g0);
            const double *X = x_ao + ((int64_t)m * n1 + g0) * nA2;  // (a, b, g) of this block
            if (!dev) {
                CUTC_CUDA_TRY(cudaMemcpyAsync(Xin, X, (size_t)gb * nA2 * 8, cudaMemcpyHostToDevice, st));
                X = Xin;
            }
            // T(i, (b, g)) = L^T X(a, (b, g))
            CUTC_TRY(fp64_gemm(st, true, n_mo, nA * gb, nA, one, dL, nA, 0, X, nA, 0, zero, T,
                               n_mo, 0, 1));
            // Y_g = T_g R for every g of the block
            CUTC_TRY(fp64_gemm(st, false, n_mo, n_mo, nA, one, T, n_mo, (int64_t)n_mo * nA, dR,
                               nA, 0, zero, Y, n_mo, nm2, gb));
            // X_mo(g, m, (i, j)) = Y((i, j), g)
            if (dev) {
                CUTC_TRY(launch_transpose(st, Y, nm2, gb, (int)nm2, x_mo + (int64_t)m * n1 + g0, ldo));
            } else {
                CUTC_TRY(launch_transpose(st, Y, nm2, gb, (int)nm2, Xout, gb));
                CUTC_CUDA_TRY(cudaMemcpy2DAsync(x_mo + (int64_t)m * n1 + g0, (size_t)ldo * 8, Xout,
                                                (size_t)gb * 8, (size_t)gb * 8, (size_t)nm2,
                                                cudaMemcpyDeviceToHost, st));
            }
        }
    }
    if (!dev)
        CUTC_CUDA_TRY(cudaStreamSynchronize(st));
    return CUTC_OK;
}

}  // namespace cutc

extern "C" int cutc_x_ao_to_mo(int n_grid1, int n_ao, int n_mo, int components,
                               const double *mo_l_coef, const double *mo_r_coef,
                               const double *x_ao, double *x_mo, int device_pointers, void *stream)
{
    using namespace cutc;
    if (n_grid1 <= 0 || n_ao <= 0 || n_mo <= 0 || (components != 3 && components != 4) ||
        !mo_l_coef || !mo_r_coef || !x_ao || !x_mo) {
        cutc_set_error(CUTC_ERR_INVALID, "invalid AO-to-MO arguments");
        return CUTC_ERR_INVALID;
    }
    if ((int64_t)n_mo * n_mo > INT32_MAX / 2 || (int64_t)n_ao * n_ao > INT32_MAX / 2) {
        cutc_set_error(CUTC_ERR_INVALID, "n_ao or n_mo too large");
        return CUTC_ERR_INVALID;
    }
    Engine *E = nullptr;
    CUTC_TRY(get_engine(&E));
    std::lock_guard<std::mutex> lk(E->mu);
    cudaStream_t st = stream ? (cudaStream_t)stream : E->stream;
    int s = x_ao_to_mo(E, st, n_grid1, n_ao, n_mo, components, mo_l_coef, mo_r_coef, x_ao, x_mo,
                       device_pointers != 0, (size_t)2 << 30);
    if (s != CUTC_OK)
        cudaStreamSynchronize(st);
    return s;
}
