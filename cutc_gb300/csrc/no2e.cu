// The two-electron contraction of the reference's normal-ordering driver, on its
// intermediates (src/cutc_no.c:415-470):
//
//   no_2e = 1/2 tmpC1^T X + 1/2 tmpC2^T tmpD2      (M = N = n_mo^2, K = 3 n1 and n1)
//   no_2e <- no_2e + no_2e^T                        (trans_inplace)
//   no_2e(p, q, s, t) <- no_2e(p, s, q, t)          (trans_pqst_psqt_inplace)
//
// X is the MO-basis X in cutc_no's point-fastest order, X[(g + n1 m) + 3 n1 (i + n_mo j)],
// which cutc_x_ao_to_mo writes; tmpC1 has its layout, tmpC2 and tmpD2 are
// [g + n1 (i + n_mo j)].  The reference runs the two products as cuBLAS DGEMMs; here the
// plain form uses the FP64 DMMA GEMM (two products, the second accumulating) and the split
// form one split contraction over the concatenated K = 4 n1.  The symmetrisation and the
// index swap run on the coalesced layout kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "dgemm.cuh"
#include "engine.cuh"
#include "products.cuh"
#include "split.cuh"

namespace cutc {

enum No2eSlot { N_C1 = 220, N_X, N_C2, N_D2, N_OUT };

}  // namespace cutc

using namespace cutc;

extern "C" int cutc_no_2e(const cutc_options *opt, int n_mo, int n_grid1, const double *tmpC1,
                          const double *x_mo, const double *tmpC2, const double *tmpD2,
                          double *no_2e)
{
    cutc_options defaults;
    if (!opt) {
        cutc_default_options(&defaults);
        opt = &defaults;
    }
    const int64_t nm2 = (int64_t)n_mo * n_mo;
    if (n_mo <= 0 || n_grid1 <= 0 || !tmpC1 || !x_mo || !tmpC2 || !tmpD2 || !no_2e ||
        nm2 > INT32_MAX / 2 || n_mo > 65535 ||
        (opt->precision != CUTC_PLAIN_FP64 && opt->precision != CUTC_SPLIT_BF16) ||
        (opt->precision == CUTC_SPLIT_BF16 &&
         (opt->n_slices < 3 || opt->n_slices > kMaxSlices))) {
        cutc_set_error(CUTC_ERR_INVALID, "invalid cutc_no_2e arguments (n_mo=%d n_grid1=%d)",
                       n_mo, n_grid1);
        return CUTC_ERR_INVALID;
    }
    Engine *E = nullptr;
    CUTC_TRY(get_engine(&E));
    std::lock_guard<std::mutex> lk(E->mu);
    cudaStream_t st = opt->stream ? (cudaStream_t)opt->stream : E->stream;
    const int64_t n1 = n_grid1, k1 = 3 * n1;
    const size_t b1 = (size_t)k1 * nm2 * 8, b2 = (size_t)n1 * nm2 * 8, bo = (size_t)nm2 * nm2 * 8;
    const double *C1 = tmpC1, *X = x_mo, *C2 = tmpC2, *D2 = tmpD2;
    double *out = no_2e;
    if (!opt->device_pointers) {
        void *p;
        const struct { int slot; const double *src; size_t bytes; const double **dst; } up[] = {
            {N_C1, tmpC1, b1, &C1}, {N_X, x_mo, b1, &X}, {N_C2, tmpC2, b2, &C2},
            {N_D2, tmpD2, b2, &D2}};
        for (const auto &u : up) {
            CUTC_TRY(E->ws.get(u.slot, u.bytes, &p));
            CUTC_CUDA_TRY(cudaMemcpyAsync(p, u.src, u.bytes, cudaMemcpyHostToDevice, st));
            *u.dst = (const double *)p;
        }
        CUTC_TRY(E->ws.get(N_OUT, bo, &p));
        out = (double *)p;
    }
    if (opt->precision == CUTC_PLAIN_FP64) {
        // no_2e = 1/2 tmpC1^T X, then += 1/2 tmpC2^T tmpD2 (src/cutc_no.c:419-446)
        CUTC_TRY(fp64_gemm(st, true, (int)nm2, (int)nm2, k1, 0.5, C1, k1, 0, X, k1, 0, 0.0, out,
                           nm2, 0, 1));
        CUTC_TRY(fp64_gemm(st, true, (int)nm2, (int)nm2, n1, 0.5, C2, n1, 0, D2, n1, 0, 1.0, out,
                           nm2, 0, 1));
    } else {
        CUTC_TRY(split_gemm_concat(E, st, opt->n_slices, (int)nm2, (int)nm2, k1, C1, X, n1, C2,
                                   D2, 0.5, out, nm2));
    }
    CUTC_TRY(launch_add_transpose(st, out, (int)nm2));  // src/cutc_no.c:457
    CUTC_TRY(launch_swap_qs(st, out, n_mo));             // src/cutc_no.c:468
    if (!opt->device_pointers)
        CUTC_CUDA_TRY(cudaMemcpyAsync(no_2e, out, bo, cudaMemcpyDeviceToHost, st));
    CUTC_CUDA_TRY(cudaStreamSynchronize(st));
    return CUTC_OK;
}
