// FP64 GEMM of the plain form: DMMA (mma.sync m8n8k4 .f64) tiles fed by a
// multi-stage cp.async pipeline.
//
// The plain form keeps every contraction of the cutc_int path in FP64, as the
// reference does with cublasDgemm (src/build_int2_grad1_u12_ao.cu:152-159,
// src/build_int_2e_ao.cu:60-67 and 97-104):
//   X_m[p, r1] = sum_r2 P[p, r2] G_m[r1, r2]        (A K-contiguous, "OP_T")
//   H[p, q]    = sum_r1 X_3[p, r1] S0[q, r1]        (A M-contiguous, "OP_N")
//   N[p, l]    = -1/2 sum_{m, r1} X_m[p, r1] S_m[l, r1]
// GB300 executes FP64 at about 2 FMA per clock per SM (1.25 TFLOP/s for the
// chip), so these contractions are bound by the FP64 pipe and nothing else:
// a 128 x 128 x 16 tile step is 262 144 FMAs, ~130 000 clocks of one SM's
// FP64 pipe, against 32 KB of operands -- 0.25 B per clock of operand
// traffic, far below every memory limit.  What the kernel needs is the FP64
// pipe never idle: eight warps per CTA, each with 32 independent DMMAs per
// 4-wide K step (a 64 x 32 warp tile, 64 FP64 accumulators per thread), and
// the next operand tiles in flight (three cp.async stages) while the current
// one is consumed.  Operands are copied with 8-byte cp.async, whose only
// alignment rule is the element's own: the strides here (n_grid2, block
// rows, n_ao^2) are arbitrary, which rules out TMA's 16-byte stride rule, and
// the copy engine would buy nothing at this arithmetic intensity.
//
// Shared-memory tiles are padded so that the DMMA fragment loads (8 rows x 4 k
// per warp, 256 bytes) take the minimum two wavefronts: a K-contiguous
// operand is stored [row][k] with 20 doubles per row, an M-contiguous one
// [k][row] with 136 doubles per k.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>

#include "common.cuh"
#include "dgemm.cuh"

namespace cutc {

namespace {

constexpr int kBM = 128, kBN = 128, kBK = 16, kStages = 3, kThreads = 256;
constexpr int kLdRow = kBK + 4;               // [row][k] tiles
constexpr int kLdCol = kBM + 8;               // [k][row] tiles
constexpr int kTileRow = kBM * kLdRow;        // 2560 doubles
constexpr int kTileCol = kBK * kLdCol;        // 2176 doubles
constexpr int kStageA = kTileRow > kTileCol ? kTileRow : kTileCol;
constexpr int kStageB = kBN * kLdRow;
constexpr int kSmem = kStages * (kStageA + kStageB) * (int)sizeof(double);  // 120 KB
static_assert(kBM == kBN, "the loaders assume square CTA tiles");

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// 8-byte asynchronous copy; src_bytes = 0 writes zeros (out-of-range elements)
__device__ __forceinline__ void cp_async8(uint32_t dst, const double *src, uint32_t src_bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src),
                 "r"(src_bytes)
                 : "memory");
}

__device__ __forceinline__ void cp_async_commit()
{
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// d += a b over one 8 x 8 x 4 step: a = A[lane / 4][lane % 4] (row-major A),
// b = B[lane % 4][lane / 4] (column-major B), d = D[lane / 4][2 (lane % 4) + {0, 1}].
__device__ __forceinline__ void dmma(double &d0, double &d1, double a, double b)
{
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

struct Args {
    int M, N;
    int64_t K;
    double alpha, beta;
    const double *A, *B;
    double *C;
    int64_t lda, ldb, ldc, sa, sb, sc;
    int tiles_m, tiles_n;
};

template <bool AK>
__global__ void __launch_bounds__(kThreads, 1) fp64_gemm_kernel(const Args g)
{
    extern __shared__ __align__(16) double smem[];
    double *sA = smem;                       // kStages x kStageA
    double *sB = smem + kStages * kStageA;   // kStages x kStageB

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t per_batch = (int64_t)g.tiles_m * g.tiles_n;
    const int64_t t = blockIdx.x;
    const int z = (int)(t / per_batch);
    const int64_t r = t - (int64_t)z * per_batch;
    const int m0 = (int)(r % g.tiles_m) * kBM;  // m fastest: a wave shares the B tiles
    const int n0 = (int)(r / g.tiles_m) * kBN;
    const double *A = g.A + (int64_t)z * g.sa;
    const double *B = g.B + (int64_t)z * g.sb;
    double *C = g.C + (int64_t)z * g.sc;
    const int64_t nkb = (g.K + kBK - 1) / kBK;

    auto load = [&](int stage, int64_t kb) {
        const int64_t k0 = kb * kBK;
        double *a = sA + stage * kStageA, *b = sB + stage * kStageB;
#pragma unroll
        for (int i = 0; i < kBM * kBK / kThreads; i++) {
            const int e = tid + kThreads * i;
            int row, k;
            if (AK) {
                row = e / kBK;
                k = e % kBK;
            } else {
                k = e / kBM;
                row = e % kBM;
            }
            const int gm = m0 + row;
            const int64_t gk = k0 + k;
            const bool ok = gm < g.M && gk < g.K;
            const double *src = ok ? (AK ? A + (int64_t)gm * g.lda + gk : A + gk * g.lda + gm) : A;
            cp_async8(smem_u32(AK ? a + row * kLdRow + k : a + k * kLdCol + row), src, ok ? 8u : 0u);
        }
#pragma unroll
        for (int i = 0; i < kBN * kBK / kThreads; i++) {
            const int e = tid + kThreads * i;
            const int row = e / kBK, k = e % kBK;
            const int gn = n0 + row;
            const int64_t gk = k0 + k;
            const bool ok = gn < g.N && gk < g.K;
            const double *src = ok ? B + (int64_t)gn * g.ldb + gk : B;
            cp_async8(smem_u32(b + row * kLdRow + k), src, ok ? 8u : 0u);
        }
    };

    // warp tile: rows wm * 64 .. + 64, columns wn * 32 .. + 32
    const int wm = warp & 1, wn = warp >> 1;
    const int fr = lane >> 2, fk = lane & 3;
    double acc[8][4][2];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
            acc[i][j][0] = acc[i][j][1] = 0.0;

#pragma unroll
    for (int s = 0; s < kStages - 1; s++) {
        if (s < nkb)
            load(s, s);
        cp_async_commit();
    }
    for (int64_t kb = 0; kb < nkb; kb++) {
        cp_async_wait<kStages - 2>();
        __syncthreads();  // stage kb landed for every thread; stage kb - 1 is free
        const int64_t pre = kb + kStages - 1;
        if (pre < nkb)
            load((int)(pre % kStages), pre);
        cp_async_commit();
        const int stage = (int)(kb % kStages);
        const double *a = sA + stage * kStageA, *b = sB + stage * kStageB;
#pragma unroll
        for (int kk = 0; kk < kBK / 4; kk++) {
            const int k = kk * 4 + fk;
            double av[8], bv[4];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int row = wm * 64 + i * 8 + fr;
                av[i] = AK ? a[row * kLdRow + k] : a[k * kLdCol + row];
            }
#pragma unroll
            for (int j = 0; j < 4; j++)
                bv[j] = b[(wn * 32 + j * 8 + fr) * kLdRow + k];
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 4; j++)
                    dmma(acc[i][j][0], acc[i][j][1], av[i], bv[j]);
        }
    }
    cp_async_wait<0>();

#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int m = m0 + wm * 64 + i * 8 + fr;
        if (m >= g.M)
            continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int n = n0 + wn * 32 + j * 8 + 2 * fk + h;
                if (n < g.N) {
                    double *c = C + m + (int64_t)n * g.ldc;
                    const double v = g.alpha * acc[i][j][h];
                    *c = g.beta == 0.0 ? v : v + g.beta * *c;
                }
            }
        }
    }
}

}  // namespace

int fp64_gemm(cudaStream_t st, bool a_kmajor, int M, int N, int64_t K, double alpha,
              const double *A, int64_t lda, int64_t sa, const double *B, int64_t ldb, int64_t sb,
              double beta, double *C, int64_t ldc, int64_t sc, int batch)
{
    if (M < 0 || N < 0 || K < 0 || batch < 0 || ldc < std::max(1, M) ||
        (K > 0 && (!A || !B || ldb < K || lda < (a_kmajor ? K : (int64_t)M))) || (M && N && !C)) {
        cutc_set_error(CUTC_ERR_INVALID, "invalid FP64 GEMM arguments (M=%d N=%d K=%lld)", M, N,
                       (long long)K);
        return CUTC_ERR_INVALID;
    }
    if (M == 0 || N == 0 || batch == 0)
        return CUTC_OK;
    static std::atomic<unsigned long long> attr_done{0};
    const unsigned long long bit = current_device_bit();
    if (!(attr_done.load() & bit)) {
        CUTC_CUDA_TRY(cudaFuncSetAttribute(fp64_gemm_kernel<true>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem));
        CUTC_CUDA_TRY(cudaFuncSetAttribute(fp64_gemm_kernel<false>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem));
        attr_done.fetch_or(bit);
    }
    Args g;
    g.M = M;
    g.N = N;
    g.K = K;
    g.alpha = alpha;
    g.beta = beta;
    g.A = A;
    g.B = B;
    g.C = C;
    g.lda = lda;
    g.ldb = ldb;
    g.ldc = ldc;
    g.sa = sa;
    g.sb = sb;
    g.sc = sc;
    g.tiles_m = (M + kBM - 1) / kBM;
    g.tiles_n = (N + kBN - 1) / kBN;
    const int64_t tiles = (int64_t)g.tiles_m * g.tiles_n * batch;
    if (tiles > INT32_MAX) {
        cutc_set_error(CUTC_ERR_INVALID, "FP64 GEMM of %lld tiles exceeds one grid",
                       (long long)tiles);
        return CUTC_ERR_INVALID;
    }
    if (a_kmajor)
        fp64_gemm_kernel<true><<<(unsigned)tiles, kThreads, kSmem, st>>>(g);
    else
        fp64_gemm_kernel<false><<<(unsigned)tiles, kThreads, kSmem, st>>>(g);
    CUTC_CUDA_TRY(cudaGetLastError());
    note_launches(1);
    return CUTC_OK;
}

}  // namespace cutc
