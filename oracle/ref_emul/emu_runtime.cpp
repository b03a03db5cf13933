/*
 * Host implementation of the emulated CUDA runtime / cuBLAS calls declared in
 * emu_cuda.h -- TEST INFRASTRUCTURE ONLY (see that header).
 */
#include "emu_cuda.h"

#include <stdint.h>

dim3 blockIdx, threadIdx, blockDim, gridDim;

/* the shared-memory window of the one kernel on the path that uses it */
alignas(16) char shared_data[1 << 20];

static size_t g_free_bytes = (size_t)270 << 30; /* a GB300-sized free pool */

extern "C" {

void emu_set_free_bytes(size_t free_b) { g_free_bytes = free_b; }

cudaError_t cudaMalloc(void **p, size_t n)
{
    /* deliberately not zeroed, like device memory */
    *p = malloc(n ? n : 1);
    if (*p && n) {
        /* fill with a NaN pattern so reads of unwritten memory show up */
        memset(*p, 0xff, n);
    }
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}

cudaError_t cudaFree(void *p)
{
    free(p);
    return cudaSuccess;
}

cudaError_t cudaMemcpy(void *dst, const void *src, size_t n, enum cudaMemcpyKind)
{
    memcpy(dst, src, n);
    return cudaSuccess;
}

cudaError_t cudaMemGetInfo(size_t *free_b, size_t *total_b)
{
    *free_b = g_free_bytes;
    *total_b = g_free_bytes + ((size_t)10 << 30);
    return cudaSuccess;
}

cudaError_t cudaGetDeviceProperties(struct cudaDeviceProp *prop, int)
{
    memset(prop, 0, sizeof(*prop));
    strcpy(prop->name, "host emulation");
    prop->maxThreadsPerBlock = 1024;
    prop->maxThreadsDim[0] = 1024;
    prop->maxThreadsDim[1] = 1024;
    prop->maxThreadsDim[2] = 64;
    prop->maxGridSize[0] = 2147483647;
    prop->maxGridSize[1] = 65535;
    prop->maxGridSize[2] = 65535;
    return cudaSuccess;
}

cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
const char *cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "error"; }

struct emu_event { int dummy; };
cudaError_t cudaEventCreate(cudaEvent_t *e)
{
    *e = (cudaEvent_t)malloc(sizeof(struct emu_event));
    return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t, int) { return cudaSuccess; }
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t, cudaEvent_t)
{
    *ms = 0.0f;
    return cudaSuccess;
}
cudaError_t cudaEventDestroy(cudaEvent_t e)
{
    free(e);
    return cudaSuccess;
}

struct emu_cublas { int dummy; };
cublasStatus_t cublasCreate(cublasHandle_t *h)
{
    *h = (cublasHandle_t)malloc(sizeof(struct emu_cublas));
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasDestroy(cublasHandle_t h)
{
    free(h);
    return CUBLAS_STATUS_SUCCESS;
}

/* Column-major C = alpha op(A) op(B) + beta C with BLAS semantics (beta == 0
 * overwrites C without reading it). */
cublasStatus_t cublasDgemm(cublasHandle_t, cublasOperation_t ta, cublasOperation_t tb,
                           int m, int n, int k, const double *alpha,
                           const double *A, int lda, const double *B, int ldb,
                           const double *beta, double *C, int ldc)
{
    const double al = *alpha, be = *beta;
#pragma omp parallel for schedule(dynamic, 1)
    for (int j = 0; j < n; j++) {
        double *acc = (double *)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
        for (int i = 0; i < m; i++)
            acc[i] = 0.0;
        for (int l = 0; l < k; l++) {
            const double b = (tb == CUBLAS_OP_N) ? B[l + (int64_t)ldb * j] : B[j + (int64_t)ldb * l];
            if (ta == CUBLAS_OP_N) {
                const double *a = A + (int64_t)lda * l;
                for (int i = 0; i < m; i++)
                    acc[i] += a[i] * b;
            } else {
                for (int i = 0; i < m; i++)
                    acc[i] += A[l + (int64_t)lda * i] * b;
            }
        }
        for (int i = 0; i < m; i++) {
            double *c = C + i + (int64_t)ldc * j;
            *c = (be == 0.0) ? al * acc[i] : al * acc[i] + be * *c;
        }
        free(acc);
    }
    return CUBLAS_STATUS_SUCCESS;
}

} /* extern "C" */
