/*
 * Host emulation of the small CUDA runtime / cuBLAS surface that the
 * reference's cutc_int path uses -- TEST INFRASTRUCTURE ONLY.
 *
 * With these declarations the reference sources compile with gcc/g++ and run
 * on the CPU: device memory is host memory, copies are memcpy, cuBLAS DGEMM is
 * a plain FP64 loop, and a kernel launch runs every (block, thread) of the
 * launch grid one after another.  That is exact for the reference kernels on
 * this path: the only cross-thread traffic is the shared-memory staging in
 * jast_bh.cu:91-107, where every thread writes identical values before use.
 *
 * Used only by oracle/ref_emul/build_ref.py to produce oracle/_ref/, which in
 * turn only generates the golden fixtures under tests/golden/.
 */
#ifndef CUTC_EMU_CUDA_H
#define CUTC_EMU_CUDA_H

#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum cudaError_enum_emu {
    cudaSuccess = 0,
    cudaErrorMemoryAllocation = 2,
    cudaErrorInvalidValue = 1
} cudaError_t;

enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3,
    cudaMemcpyDefault = 4
};

struct dim3 {
    unsigned int x, y, z;
#ifdef __cplusplus
    dim3(unsigned int vx = 1, unsigned int vy = 1, unsigned int vz = 1) : x(vx), y(vy), z(vz) {}
#endif
};
#ifndef __cplusplus
typedef struct dim3 dim3;
#endif

struct cudaDeviceProp {
    char name[256];
    int maxThreadsPerBlock;
    int maxThreadsDim[3];
    int maxGridSize[3];
};

typedef struct emu_event *cudaEvent_t;

cudaError_t cudaMalloc(void **p, size_t n);
cudaError_t cudaFree(void *p);
cudaError_t cudaMemcpy(void *dst, const void *src, size_t n, enum cudaMemcpyKind k);
cudaError_t cudaMemGetInfo(size_t *free_b, size_t *total_b);
cudaError_t cudaGetDeviceProperties(struct cudaDeviceProp *prop, int dev);
cudaError_t cudaDeviceSynchronize(void);
cudaError_t cudaGetLastError(void);
const char *cudaGetErrorString(cudaError_t e);
cudaError_t cudaEventCreate(cudaEvent_t *e);
cudaError_t cudaEventRecord(cudaEvent_t e, int stream);
cudaError_t cudaEventSynchronize(cudaEvent_t e);
cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t a, cudaEvent_t b);
cudaError_t cudaEventDestroy(cudaEvent_t e);

typedef enum {
    CUBLAS_STATUS_SUCCESS = 0,
    CUBLAS_STATUS_NOT_INITIALIZED = 1,
    CUBLAS_STATUS_ALLOC_FAILED = 3,
    CUBLAS_STATUS_INVALID_VALUE = 7,
    CUBLAS_STATUS_ARCH_MISMATCH = 8,
    CUBLAS_STATUS_MAPPING_ERROR = 11,
    CUBLAS_STATUS_EXECUTION_FAILED = 13,
    CUBLAS_STATUS_INTERNAL_ERROR = 14,
    CUBLAS_STATUS_NOT_SUPPORTED = 15,
    CUBLAS_STATUS_LICENSE_ERROR = 16
} cublasStatus_t;

typedef enum { CUBLAS_OP_N = 0, CUBLAS_OP_T = 1, CUBLAS_OP_C = 2 } cublasOperation_t;

typedef struct emu_cublas *cublasHandle_t;

cublasStatus_t cublasCreate(cublasHandle_t *h);
cublasStatus_t cublasDestroy(cublasHandle_t h);
cublasStatus_t cublasDgemm(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb,
                           int m, int n, int k, const double *alpha,
                           const double *A, int lda, const double *B, int ldb,
                           const double *beta, double *C, int ldc);

/* free-memory figure reported to the reference's tiling code */
void emu_set_free_bytes(size_t free_b);

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
/* ---- device-side emulation (C++ translation units only) ---- */
#define __global__
#define __device__
#define __host__
#define __shared__
#define __forceinline__ inline

extern dim3 blockIdx, threadIdx, blockDim, gridDim;

static inline double __int2double_rn(int v) { return (double)v; }
static inline void __syncthreads(void) {}

template <class F>
static void emu_launch(dim3 g, dim3 b, size_t /*smem*/, F f)
{
    gridDim = g;
    blockDim = b;
    for (unsigned bz = 0; bz < g.z; bz++)
        for (unsigned by = 0; by < g.y; by++)
            for (unsigned bx = 0; bx < g.x; bx++)
                for (unsigned tz = 0; tz < b.z; tz++)
                    for (unsigned ty = 0; ty < b.y; ty++)
                        for (unsigned tx = 0; tx < b.x; tx++) {
                            blockIdx = dim3(bx, by, bz);
                            threadIdx = dim3(tx, ty, tz);
                            f();
                        }
}

template <class F>
static void emu_launch(dim3 g, dim3 b, F f)
{
    emu_launch(g, b, 0, f);
}
#endif

#endif
