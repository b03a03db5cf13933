// Split-precision contractions on the sm_103a tensor cores (tcgen05 + TMA).
//
// Both dense contractions of the cutc_int path
//   X_m[p, r1] = sum_r2 P[p, r2] G_m[r1, r2]                    (X build)
//   H[p, q] = sum_r1 X_3[p, r1] S0[q, r1],
//   N[p, l] = -1/2 sum_{m, r1} X_m[p, r1] S_m[l, r1]          (int_2e)
// are C[M x N] = alpha * A[M x K] B[N x K]^T with FP64 operands.  Each FP64
// operand row r is written as
//     A[r, k] = 2^{e_r} sum_{s < S} a_s[r, k],  a_s = q_s 2^{-8-9s},  q_s in [-256, 256]
// (S signed 9-bit digits of the row-scaled value, rounded at the last digit:
// relative error <= 2^{-9S}), and every digit is an exact BF16 number.  The
// products a_s b_t with s + t <= D = S - 1 run as tcgen05.mma kind::f16 (BF16
// in, FP32 accumulate in tensor memory), one accumulator per diagonal d = s + t:
//   * the accumulator of diagonal d sits at tensor-memory column BN d, so the
//     products of slice a_s with b_0 .. b_{D-s} -- the B slices stacked in
//     shared memory -- are ONE instruction of width N = BN (D + 1 - s) that
//     lands on diagonals s .. D: S instructions per 16-wide K step instead of
//     S (S + 1) / 2, and A is read from shared memory once per slice, which
//     keeps the operand traffic under the shared-memory bandwidth;
//   * every product of diagonal d is an integer multiple of 2^{-16-9d} of
//     magnitude <= 2^{-9d}, so the FP32 accumulator holds the exact sum while
//     (d + 1) * Kc * 2^16 <= 2^24.  The chunk is Kc = 128: exact for d <= 1;
//     diagonal 2 (3 * 128 * 2^16 = 1.5 * 2^24 quanta at most) can round only if
//     a chunk sum of 384 remainder-digit products exceeds 2^24 quanta, and then
//     by one quantum 2^-34, which over the whole K stays below 2^-41 of
//     sum_k |a_k b_k| -- under the slicing's own representation error.  (Kc = 64
//     keeps d = 2 provably exact but flushes twice as often: 9 % slower on the
//     medium X contraction at the same measured error);
//   * after each chunk the epilogue adds the d = 0, 1, 2 sums error-free into
//     FP32 (hi, lo) register pairs (hi on a coarse grid, lo the remainder)
//     and d >= 3 (relative size 2^-27) into a plain FP32 sum; nothing is
//     carried across chunks in tensor memory, whose FP32 accumulation
//     rounding would otherwise grow with K;
//   * the accumulators are double-buffered in tensor memory, so the flush of
//     chunk c overlaps the MMAs of chunk c + 1;
//   * at the end the seven FP32 pieces are summed error-free (TwoSum on f32x2 pairs
//     of columns, the small remainders in FP32), the double-float result is
//     converted with one FP64 add, and the scale 2^{e_r + f_n} (and a power-of-two
//     alpha) is added to the exponent bits.
// FP64 arithmetic is used only in that conversion (and in the pair terms that feed
// G): GB300's FP64 pipe runs at 1/64 of the FP32 rate, and a full FP64 sum of the
// pieces cost 7 % of the contraction.
// The scheme is the error-free splitting of Ozaki, Ogita, Oishi & Rump
// (2012), on BF16 instead of FP64 slices, with exact FP32 chunk accumulation.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstdlib>
#include <vector>

#include "common.cuh"
#include "dfloat.cuh"
#include "digits.cuh"
#include "pair.cuh"
#include "products.cuh"
#include "split.cuh"
#include "tc.cuh"

namespace cutc {

// ---------------------------------------------------------------------------
// GEMM kernel
// ---------------------------------------------------------------------------

constexpr int kBM = 128;        // rows of A per CTA (TMEM lanes)
constexpr int kBK = 32;         // K per TMA box: 32 BF16 = 64-byte rows (64B swizzle)
constexpr int kChunkBlocks = 4; // exact-accumulation chunk: 128 K
constexpr int kMaxKPerLaunch = 1 << 18;  // keeps every exact (hi, lo) sum below 2^24 units
// Default K per launch: one launch up to kLongK; a longer contraction runs as equal
// launches of at most kLaunchK, summed in FP64 (the C += epilogue).  On one GB300 the
// X contraction of the 300-AO molecule (K = 200 000, 1500 r1 rows) took 1826 ms in one
// launch and 1282 ms in five of 40 000; the medium one (K = 80 000) 1176 and 1168 ms
// in one and two launches, and 1205 ms in three.  Over a long K loop the CTAs of a
// wave probably drift apart and stop sharing their A and B tiles in L2.  With an A
// operand of kBigM rows or more, launches of at most kLaunchKBigM pay: the 300-AO X
// contraction (M = 45 150, K = 200 000) took 5141 ms per 6000 r1 rows in launches of
// 40 000, 4995 in launches of 20 000 and 4971 in launches of 10 000, while the medium
// one (M = 7260) was the same at 40 000 and 20 000 and 4 % slower at 10 000.
constexpr int kLongK = 65536;
constexpr int kLaunchK = 49152;
constexpr int kBigM = 16384;
constexpr int kLongKBigM = 32768;
constexpr int kLaunchKBigM = 24576;
constexpr uint32_t kTmemCols = 512;
constexpr int kGroupN = 8;      // column tiles per raster group (B tiles shared through L2)

// Output-column tile for S slices: S diagonals x 2 buffers must fit 512 columns
// and the widest instruction (N = BN S) must not exceed 256.
__host__ __device__ constexpr int bn_for(int S) { return S <= 5 ? 48 : 32; }

struct GemmParams {
    int M, N;
    int Mpad, Npad;
    int kb0, nkb;          // K blocks [kb0, kb0 + nkb) of this launch
    const int *ea;         // row exponents of A (Mpad)
    const int *eb;         // row exponents of B (Npad)
    double alpha;          // result x 2^alpha_exp, negated if alpha_neg, x alpha if alpha_mul
    int alpha_exp, alpha_neg, alpha_mul;
    double *C;
    int64_t ldc;           // C[m + ldc * col(n)]
    int ncol_group;        // col(n) = (n / ncol_group) * group_stride + col0 + n % ncol_group
    int64_t group_stride;
    int64_t col0;
    int accumulate;        // C += result
    int *err;              // set to a non-zero code if a bounded wait gave up
};

template <int S>
struct GemmCfg {
    static constexpr int kBN = bn_for(S);
    static constexpr int kCW = 8;                    // columns per epilogue warp
    static constexpr int kEpiWarps = 4 * (kBN / kCW); // 4 lane quarters x column groups
    static constexpr int kTmaWarp = kEpiWarps;
    static constexpr int kMmaWarp = kEpiWarps + 1;
    static constexpr int kThreads = (kEpiWarps + 2) * 32;
    static constexpr int kBuf = kBN * S;             // tensor-memory columns per buffer
    static constexpr int kASlice = kBM * kBK * 2;
    static constexpr int kBSlice = kBN * kBK * 2;
    static constexpr int kStage = S * (kASlice + kBSlice);
    static constexpr int kStagesFit = (220 * 1024) / kStage;
    static constexpr int kStages = kStagesFit < 4 ? kStagesFit : 4;
    static constexpr int kBarBytes = 256;
    static constexpr int kSmem = kStages * kStage + 1024 + kBarBytes;
    static_assert(kStages >= 2, "not enough shared memory for two stages");
    static_assert(2 * kBuf <= (int)kTmemCols, "accumulators exceed tensor memory");
    static_assert(kBN * S <= 256, "instruction N exceeds 256");
    static_assert(kBSlice % 512 == 0, "B slices must stack on 8-row swizzle atoms");
};

__device__ __forceinline__ double pow2(int e)
{
    e = e < -1022 ? -1022 : (e > 1023 ? 1023 : e);
    return __longlong_as_double((long long)(1023 + e) << 52);
}

// v 2^k: the exponent field moved with integer operations when v and the result are
// normal numbers (GB300's FP64 pipe is slow), scalbn otherwise (zeros, and results that
// underflow to subnormals or zero or overflow to infinity)
__device__ __forceinline__ double scale_pow2(double v, int k)
{
    const long long b = __double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e != 0 && e + k >= 1 && e + k <= 2046)
        return __longlong_as_double(b + ((long long)k << 52));
    return scalbn(v, k);
}

template <int S>
__global__ void __launch_bounds__(GemmCfg<S>::kThreads, 1)
split_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                  GemmParams P)
{
    using Cfg = GemmCfg<S>;
    constexpr int D = S - 1;  // highest diagonal kept
    constexpr int BN = Cfg::kBN, CW = Cfg::kCW;
    constexpr int kEpiWarps = Cfg::kEpiWarps, kTmaWarp = Cfg::kTmaWarp, kMmaWarp = Cfg::kMmaWarp;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + Cfg::kStages * Cfg::kStage);
    uint64_t *full = bars;
    uint64_t *empty = bars + Cfg::kStages;
    uint64_t *tfull = bars + 2 * Cfg::kStages;
    uint64_t *tempty = tfull + 2;
    uint64_t *drain = tempty + 2;
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(drain + 1);
    volatile int *s_abort = reinterpret_cast<volatile int *>(s_tmem + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // grouped raster: a group of kGroupN column tiles sweeps the row tiles, so the
    // CTAs of a wave share their B tiles and a few A tiles through L2 (0.4-1% faster
    // than groups of 8 row tiles sweeping the columns, on the large and medium X builds)
    const int num_m = P.Mpad / kBM, num_n = P.Npad / BN;
    const int tid = blockIdx.x;
    const int per_group = kGroupN * num_m;
    const int gfirst = (tid / per_group) * kGroupN;
    const int gsize = min(num_n - gfirst, kGroupN);
    const int n0 = (gfirst + (tid % per_group) % gsize) * BN;
    const int m0 = ((tid % per_group) / gsize) * kBM;
    const int nkb = P.nkb;
    const int nch = (nkb + kChunkBlocks - 1) / kChunkBlocks;

    if (threadIdx.x == 0) {
        for (int i = 0; i < Cfg::kStages; i++) {
            tc::mbar_init(tc::smem_u32(&full[i]), 1);
            tc::mbar_init(tc::smem_u32(&empty[i]), 1);
        }
        for (int i = 0; i < 2; i++) {
            tc::mbar_init(tc::smem_u32(&tfull[i]), 1);
            tc::mbar_init(tc::smem_u32(&tempty[i]), kEpiWarps);
        }
        tc::mbar_init(tc::smem_u32(drain), 1);
        *s_abort = 0;
        tc::fence_mbar_init();
    }
    if (warp == kMmaWarp) {
        tc::tmem_alloc(tc::smem_u32(s_tmem), kTmemCols);
        tc::tmem_relinquish();
    }
    if (warp == kTmaWarp && lane == 0) {
        tc::tma_prefetch(&tmA);
        tc::tma_prefetch(&tmB);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *s_tmem;

    auto fail = [&](int code) {
        *s_abort = 1;
        atomicExch(P.err, code);
    };

    if (warp == kTmaWarp) {
        if (lane == 0) {
            int issued = 0;
            for (int kb = 0; kb < nkb; kb++) {
                const int stage = kb % Cfg::kStages, round = kb / Cfg::kStages;
                if (round > 0 &&
                    !tc::mbar_wait(tc::smem_u32(&empty[stage]), (round - 1) & 1, s_abort)) {
                    fail(1);
                    break;
                }
                const uint32_t fb = tc::smem_u32(&full[stage]);
                tc::mbar_arrive_expect_tx(fb, Cfg::kStage);
                uint8_t *st = smem + stage * Cfg::kStage;
                const int x = (P.kb0 + kb) * kBK;
#pragma unroll
                for (int s = 0; s < S; s++)
                    tc::tma_load_2d(tc::smem_u32(st + s * Cfg::kASlice), &tmA, x, s * P.Mpad + m0, fb);
#pragma unroll
                for (int t = 0; t < S; t++)
                    tc::tma_load_2d(tc::smem_u32(st + S * Cfg::kASlice + t * Cfg::kBSlice), &tmB, x,
                                    t * P.Npad + n0, fb);
                issued = kb + 1;
            }
            if (*s_abort) {
                // let the copies already issued land before the CTA goes away
                for (int kb = max(0, issued - Cfg::kStages); kb < issued; kb++)
                    tc::mbar_wait(tc::smem_u32(&full[kb % Cfg::kStages]),
                                  (kb / Cfg::kStages) & 1, nullptr);
            }
        }
    } else if (warp == kMmaWarp) {
        if (lane == 0) {
            bool ok = true;
            for (int c = 0; c < nch && ok; c++) {
                const int b = c & 1;
                if (c >= 2 && !tc::mbar_wait(tc::smem_u32(&tempty[b]), ((c >> 1) - 1) & 1, s_abort)) {
                    fail(2);
                    break;
                }
                tc::fence_after_sync();
                bool first = true;
                const int kb_end = min(nkb, (c + 1) * kChunkBlocks);
                for (int kb = c * kChunkBlocks; kb < kb_end; kb++) {
                    const int stage = kb % Cfg::kStages, round = kb / Cfg::kStages;
                    if (!tc::mbar_wait(tc::smem_u32(&full[stage]), round & 1, s_abort)) {
                        fail(3);
                        ok = false;
                        break;
                    }
                    tc::fence_after_sync();
                    const uint32_t sa = tc::smem_u32(smem + stage * Cfg::kStage);
                    const uint32_t sb = sa + S * Cfg::kASlice;
#pragma unroll
                    for (int k16 = 0; k16 < kBK / 16; k16++) {
                        const uint64_t bd = tc::smem_desc_sw64(sb + k16 * 32);
#pragma unroll
                        for (int s = 0; s < S; s++) {
                            // a_s x [b_0 .. b_{D-s}] -> diagonals s .. D
                            const uint32_t idesc = tc::idesc_bf16_f32(kBM, BN * (D + 1 - s));
                            const uint64_t ad = tc::smem_desc_sw64(sa + s * Cfg::kASlice + k16 * 32);
                            tc::mma_bf16(tbase + (uint32_t)(Cfg::kBuf * b + BN * s), ad, bd, idesc,
                                         first ? 0u : 1u);
                            first = false;
                        }
                    }
                    tc::mma_commit(tc::smem_u32(&empty[stage]));
                }
                if (ok)
                    tc::mma_commit(tc::smem_u32(&tfull[b]));
            }
            // all MMAs of this CTA have completed once the drain barrier flips
            tc::mma_commit(tc::smem_u32(drain));
            if (!tc::mbar_wait(tc::smem_u32(drain), 0, nullptr))
                fail(5);
        }
    } else {
        // ---- epilogue: exact chunk flushes, then the error-free final sum ----
        const int q = warp & 3, cgrp = warp >> 2;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        const uint32_t coff = (uint32_t)(CW * cgrp);
        // column pairs packed in 64 bits: every add below is one f32x2 instruction for
        // two columns (round to nearest in each lane, as the scalar form)
        constexpr int CP = CW / 2;
        uint64_t hi0[CP], lo0[CP], hi1[CP], lo1[CP], hi2[CP], lo2[CP], s3[CP];
#pragma unroll
        for (int j = 0; j < CP; j++)
            hi0[j] = lo0[j] = hi1[j] = lo1[j] = hi2[j] = lo2[j] = s3[j] = 0ull;
        // v + C - C rounds v to the grid of C's binade: C = 1.5 2^(23 + g) gives multiples of 2^g
        const uint64_t C0 = tc::f2_pack(__float_as_uint(786432.0f), __float_as_uint(786432.0f));
        // 1.5 * 2^19: multiples of 2^-4  (d = 0, LSB 2^-16)
        const uint64_t C1 = tc::f2_pack(__float_as_uint(1536.0f), __float_as_uint(1536.0f));
        // 1.5 * 2^10: multiples of 2^-13 (d = 1, LSB 2^-25)
        const uint64_t C2 = tc::f2_pack(__float_as_uint(3.0f), __float_as_uint(3.0f));
        // 1.5 * 2^1:  multiples of 2^-22 (d = 2, LSB 2^-34)
        auto exact_add = [](uint64_t x, uint64_t Cg, uint64_t &hi, uint64_t &lo) {
            const uint64_t hh = tc::f2_sub(tc::f2_add(x, Cg), Cg);
            hi = tc::f2_add(hi, hh);
            lo = tc::f2_add(lo, tc::f2_sub(x, hh));
        };
        bool ok = true;
        for (int c = 0; c < nch; c++) {
            const int b = c & 1;
            if (!tc::mbar_wait(tc::smem_u32(&tfull[b]), (c >> 1) & 1, s_abort)) {
                fail(4);
                ok = false;
                break;
            }
            tc::fence_after_sync();
#pragma unroll
            for (int h = 0; h < CW / 4; h++) {
                const uint32_t cb = tbase + lane_off + (uint32_t)(Cfg::kBuf * b) + coff + 4u * h;
                uint32_t v[4];
                tc::tmem_ld4_nowait(cb, v);
                tc::tmem_wait_ld();
                exact_add(tc::f2_pack(v[0], v[1]), C0, hi0[2 * h], lo0[2 * h]);
                exact_add(tc::f2_pack(v[2], v[3]), C0, hi0[2 * h + 1], lo0[2 * h + 1]);
                tc::tmem_ld4_nowait(cb + BN, v);
                tc::tmem_wait_ld();
                exact_add(tc::f2_pack(v[0], v[1]), C1, hi1[2 * h], lo1[2 * h]);
                exact_add(tc::f2_pack(v[2], v[3]), C1, hi1[2 * h + 1], lo1[2 * h + 1]);
                if (D >= 2) {
                    tc::tmem_ld4_nowait(cb + 2 * BN, v);
                    tc::tmem_wait_ld();
                    exact_add(tc::f2_pack(v[0], v[1]), C2, hi2[2 * h], lo2[2 * h]);
                    exact_add(tc::f2_pack(v[2], v[3]), C2, hi2[2 * h + 1], lo2[2 * h + 1]);
                }
#pragma unroll
                for (int d = 3; d <= D; d++) {
                    tc::tmem_ld4_nowait(cb + d * BN, v);
                    tc::tmem_wait_ld();
                    s3[2 * h] = tc::f2_add(s3[2 * h], tc::f2_pack(v[0], v[1]));
                    s3[2 * h + 1] = tc::f2_add(s3[2 * h + 1], tc::f2_pack(v[2], v[3]));
                }
            }
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0)
                tc::mbar_arrive(tc::smem_u32(&tempty[b]));
        }
        const int m = m0 + q * 32 + lane;
        if (ok && m < P.M) {
            const int em = P.ea[m];
            // The seven exact FP32 parts of each column, two columns per f32x2 operation:
            // hi0 + hi1 + lo0 + hi2 + lo1 by TwoSum (exact), the rounding errors and the
            // small lo2 and s3 in FP32 (below 2^-46 of the total), then one conversion to
            // FP64 per part and one FP64 add.  The power-of-two scale goes into the
            // exponent bits: GB300's FP64 pipe is slow, so the epilogue keeps off it.
            auto two_sum = [](uint64_t a, uint64_t b, uint64_t &e) -> uint64_t {
                const uint64_t sm = tc::f2_add(a, b);
                const uint64_t bb = tc::f2_sub(sm, a);
                e = tc::f2_add(tc::f2_sub(a, tc::f2_sub(sm, bb)), tc::f2_sub(b, bb));
                return sm;
            };
#pragma unroll
            for (int k = 0; k < CP; k++) {
                uint64_t e1, e2, e3, e4;
                uint64_t sm = two_sum(hi0[k], hi1[k], e1);
                sm = two_sum(sm, lo0[k], e2);
                sm = two_sum(sm, hi2[k], e3);
                sm = two_sum(sm, lo1[k], e4);
                const uint64_t lo = tc::f2_add(tc::f2_add(tc::f2_add(e1, e2), tc::f2_add(e3, e4)),
                                               tc::f2_add(lo2[k], s3[k]));
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int n = n0 + (int)coff + 2 * k + h;
                    if (n >= P.N)
                        continue;
                    const float sh = h ? tc::f2_hi(sm) : tc::f2_lo(sm);
                    const float sl = h ? tc::f2_hi(lo) : tc::f2_lo(lo);
                    double val = scale_pow2((double)sh + (double)sl, em + P.eb[n] + P.alpha_exp);
                    if (P.alpha_neg)
                        val = __longlong_as_double(__double_as_longlong(val) ^ (1ll << 63));
                    if (P.alpha_mul)
                        val *= P.alpha;
                    const int64_t col = (int64_t)(n / P.ncol_group) * P.group_stride + P.col0 +
                                        n % P.ncol_group;
                    double *dst = P.C + m + P.ldc * col;
                    *dst = P.accumulate ? *dst + val : val;
                }
            }
        }
    }

    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == kMmaWarp)
        tc::tmem_dealloc(tbase, kTmemCols);
}


// ---------------------------------------------------------------------------
// Pair terms on the tensor cores (split form, Jastrow exponents in {0, 2, 3, 4})
//
// The nucleus sum of grad1 u(r1, r2) is, for fixed g12, the contraction
//   V_c(r1, r2) = sum_k C[(r1, c)][k] F[r2][k],  k = 4 A + q over (nucleus, power of f2)
// (pair_df.cu builds F and the 16 coefficient rows C per r1 point in FP64).  Here it
// runs as a split contraction: A = the F slices (one 128-row tile of r2 points, all
// of K, loaded once per CTA), B = the coefficient slices (N tiles of 64 rows = four
// r1 points, streamed), one stacked-diagonal accumulator set in tensor memory.  The
// tensor-core work of a tile is about 1/40 of its epilogue, so one accumulator set and
// one B stage suffice: the next tile's MMAs run as soon as the epilogue has read the
// accumulators, long before it needs them, and one control warp issues both the TMA
// loads and the MMAs, which leaves registers for 16 epilogue warps (4 per SM
// sub-partition) to hide the latency of their dependent double-float chains.
// K = 4 n_nuc <= 80, so every diagonal sum is one chunk:
// diagonals 0..2 are exact in FP32 ((d + 1) * 80 * 2^16 < 2^24), d >= 3 are 2^-27 and
// below, where FP32 rounding is immaterial.
//
// The epilogue warps (lane = r2 point, one r1 point per warp) read the S diagonals
// of the point's 16 columns, add them exactly on fixed grids into double-float
// values, release the accumulators, then finish the pair in double-float exactly as
// pair_df_kernel does: g12 and its gradient, the powers of
// g, -1/2 |grad u|^2, the FP64 path near e-e coalescence, the (hi, lo) G planes and
// the G row maxima for the slicer.  Per pair that is about 800 FP32 operations
// instead of 30 df multiply-adds (~450 operations) per nucleus.
// ---------------------------------------------------------------------------

struct PairTcParams {
    int tiles_m, tiles_n, chunk;  // r2 tiles of 128 points, N tiles, N tiles per CTA
    int Mpad, Npad;               // padded rows of the F and coefficient slices
    const int *ea;                // row exponents of the F slices
    const float *bscale;          // 2^(row exponent) of each coefficient row
    const float2 *r1d;            // the tile's r1 points in double-float, [3 i + c]
    PairDfArgs P;                 // geometry, near-coalescence path and outputs
    int *err;
};

// bscale[r] = 2^ex[r] as a float
__global__ void exp_scale_kernel(const int *__restrict__ ex, int rows, float *__restrict__ bscale)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < rows) {
        const int e = max(-126, min(127, ex[r]));
        bscale[r] = __int_as_float((e + 127) << 23);
    }
}

constexpr int kPairBN = 64;  // coefficient rows per N tile: four r1 points x 16 columns

template <int S, int KB>
struct PairTcCfg {
    static constexpr int kBN = kPairBN;
    static constexpr int kPts = kBN / 16;
    static constexpr int kEpiWarps = 4 * kPts;       // lane quarter x r1 point
    static constexpr int kCtlWarp = kEpiWarps;       // TMA loads and MMAs, lane 0
    static constexpr int kThreads = (kEpiWarps + 1) * 32;
    static constexpr int kASlice = kBM * kBK * 2;
    static constexpr int kBSlice = kBN * kBK * 2;
    static constexpr int kABytes = KB * S * kASlice;
    static constexpr int kBStage = KB * S * kBSlice;
    static constexpr int kSmem = kABytes + kBStage + 1024 + 256;
    static constexpr int kMaxN = 256;                // widest kind::f16 instruction at M = 128
    static_assert(kSmem <= 227 * 1024, "shared memory");
    static_assert(kBN * S <= (int)kTmemCols, "accumulators exceed tensor memory");
    static_assert(kMaxN % kBN == 0, "instruction splits on diagonal boundaries");
    static_assert(kBSlice % 512 == 0, "B slices must stack on 8-row swizzle atoms");
    // 17 warps: the compiler's register budget is 96 per thread (it rounds the warps of
    // a CTA up when it divides the register file)
    static_assert(kThreads <= 1024, "threads per CTA");
};

// x 2^e for the scale of a value of row exponents e (clamped to the float range)
__device__ __forceinline__ float pow2f(int e)
{
    e = e < -126 ? -126 : (e > 127 ? 127 : e);
    return __int_as_float((e + 127) << 23);
}

template <int S, int KB>
__global__ void __launch_bounds__(PairTcCfg<S, KB>::kThreads, 1)
pair_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               const __grid_constant__ PairTcParams Q)
{
    using Cfg = PairTcCfg<S, KB>;
    constexpr int D = S - 1, BN = Cfg::kBN;
    constexpr int kEpiWarps = Cfg::kEpiWarps, kCtlWarp = Cfg::kCtlWarp;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint8_t *sA = smem;
    uint8_t *sB = smem + Cfg::kABytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(sB + Cfg::kBStage);
    uint64_t *afull = bars;      // the F tile has landed
    uint64_t *full = bars + 1;   // the B stage holds tile q
    uint64_t *empty = bars + 2;  // the MMAs of tile q are done with the B stage
    uint64_t *tfull = bars + 3;  // the accumulators hold tile q
    uint64_t *tempty = bars + 4; // every epilogue warp has read tile q's accumulators
    uint64_t *drain = bars + 5;
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(drain + 1);
    volatile int *s_abort = reinterpret_cast<volatile int *>(s_tmem + 1);

    const PairDfArgs &P = Q.P;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = (int)(blockIdx.x % Q.tiles_m) * kBM;
    const int t_begin = (int)(blockIdx.x / Q.tiles_m) * Q.chunk;
    const int ntiles = min(Q.tiles_n, t_begin + Q.chunk) - t_begin;

    if (threadIdx.x == 0) {
        for (int i = 0; i < 5; i++)
            tc::mbar_init(tc::smem_u32(&bars[i]), i == 4 ? kEpiWarps : 1);
        tc::mbar_init(tc::smem_u32(drain), 1);
        *s_abort = 0;
        tc::fence_mbar_init();
    }
    if (warp == kCtlWarp) {
        tc::tmem_alloc(tc::smem_u32(s_tmem), kTmemCols);
        tc::tmem_relinquish();
        if (lane == 0) {
            tc::tma_prefetch(&tmA);
            tc::tma_prefetch(&tmB);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *s_tmem;

    auto fail = [&](int code) {
        *s_abort = 1;
        atomicExch(Q.err, code);
    };

    if (warp == kCtlWarp) {
        if (lane == 0) {
            auto load_b = [&](int q) {
                const uint32_t fb = tc::smem_u32(full);
                tc::mbar_arrive_expect_tx(fb, Cfg::kBStage);
                const int n0 = (t_begin + q) * BN;
#pragma unroll
                for (int kb = 0; kb < KB; kb++)
#pragma unroll
                    for (int t = 0; t < S; t++)
                        tc::tma_load_2d(tc::smem_u32(sB + (kb * S + t) * Cfg::kBSlice), &tmB,
                                        kb * kBK, t * Q.Npad + n0, fb);
            };
            const uint32_t ab = tc::smem_u32(afull);
            tc::mbar_arrive_expect_tx(ab, Cfg::kABytes);
#pragma unroll
            for (int kb = 0; kb < KB; kb++)
#pragma unroll
                for (int s = 0; s < S; s++)
                    tc::tma_load_2d(tc::smem_u32(sA + (kb * S + s) * Cfg::kASlice), &tmA, kb * kBK,
                                    s * Q.Mpad + m0, ab);
            int loaded = 0;  // B tiles issued into the stage
            if (ntiles > 0) {
                load_b(0);
                loaded = 1;
            }
            bool ok = tc::mbar_wait(ab, 0, s_abort);
            if (!ok)
                fail(12);
            for (int q = 0; q < ntiles && ok; q++) {
                // the accumulators are free once every epilogue warp has read tile q - 1
                if (q >= 1 && !tc::mbar_wait(tc::smem_u32(tempty), (q - 1) & 1, s_abort)) {
                    fail(13);
                    break;
                }
                if (!tc::mbar_wait(tc::smem_u32(full), q & 1, s_abort)) {
                    fail(14);
                    break;
                }
                tc::fence_after_sync();
                const uint32_t sb0 = tc::smem_u32(sB);
                const uint32_t sa0 = tc::smem_u32(sA);
                bool first = true;
#pragma unroll
                for (int kb = 0; kb < KB; kb++) {
#pragma unroll
                    for (int k16 = 0; k16 < kBK / 16; k16++) {
#pragma unroll
                        for (int s = 0; s < S; s++) {
                            // a_s x [b_0 .. b_{D-s}] -> diagonals s .. D, in instructions of
                            // at most kMaxN columns
                            const uint64_t ad = tc::smem_desc_sw64(
                                sa0 + (kb * S + s) * Cfg::kASlice + k16 * 32);
#pragma unroll
                            for (int t0 = 0; t0 <= D - s; t0 += Cfg::kMaxN / BN) {
                                const int nt = min(Cfg::kMaxN / BN, D - s + 1 - t0);
                                const uint64_t bd = tc::smem_desc_sw64(
                                    sb0 + (kb * S + t0) * Cfg::kBSlice + k16 * 32);
                                tc::mma_bf16(tbase + (uint32_t)(BN * (s + t0)), ad, bd,
                                             tc::idesc_bf16_f32(kBM, BN * nt), first ? 0u : 1u);
                            }
                            first = false;
                        }
                    }
                }
                tc::mma_commit(tc::smem_u32(empty));
                tc::mma_commit(tc::smem_u32(tfull));
                // refill the B stage for tile q + 1 once these MMAs have read it
                if (q + 1 < ntiles) {
                    if (!tc::mbar_wait(tc::smem_u32(empty), q & 1, s_abort)) {
                        fail(11);
                        break;
                    }
                    load_b(q + 1);
                    loaded = q + 2;
                }
            }
            tc::mma_commit(tc::smem_u32(drain));
            if (!tc::mbar_wait(tc::smem_u32(drain), 0, nullptr))
                fail(15);
            // let the copies still in flight land before the CTA goes away
            tc::mbar_wait(ab, 0, nullptr);
            if (*s_abort && loaded > 0)
                tc::mbar_wait(tc::smem_u32(full), (loaded - 1) & 1, nullptr);
        }
    } else {
        // ---- epilogue: one r1 point of each N tile, 32 r2 points ---------------------
        const int quarter = warp & 3, pt = warp >> 2;
        const uint32_t lane_off = (uint32_t)(quarter * 32) << 16;
        const int j = m0 + quarter * 32 + lane;
        const bool jok = j < P.n2;
        const int jc = jok ? j : 0;
        const float2 x2 = P.r2d[jc], y2 = P.r2d[P.n2 + jc], z2 = P.r2d[2 * (int64_t)P.n2 + jc];
        const float sa = pow2f(Q.ea[jc]);  // F rows: 2^1 (f^0 = 1 is the row maximum)
        const df::D a = df::make(P.a_ee_hi, P.a_ee_lo);
        for (int q = 0; q < ntiles; q++) {
            if (!tc::mbar_wait(tc::smem_u32(tfull), q & 1, s_abort)) {
                fail(16);
                break;
            }
            tc::fence_after_sync();
            // The point's 16 columns on each diagonal, summed exactly on grids.  In units of
            // the row scales every diagonal sum D_d is a multiple of 2^(-16-9d) and |D_0| <= K:
            //   H  = D_0 + D_1 rounded to multiples of 2^-16      (exact: below 2^7 there)
            //   L  = the rest of D_1 + D_2 rounded to 2^-25         (exact: below 2^-8 there)
            //   L2 = the rest of D_2 + D_3 + ... (FP32; below 2^-18, so off by < 2^-42)
            // Two columns share each packed f32x2 operation.
            uint64_t H[8], L[8], L2[8];
            {
                const uint32_t cb = tbase + lane_off + (uint32_t)(16 * pt);
                const uint64_t C16 = tc::f2_pack(__float_as_uint(192.0f), __float_as_uint(192.0f));
                const uint64_t C25 = tc::f2_pack(__float_as_uint(0.375f), __float_as_uint(0.375f));
                float v[16];
                tc::tmem_ld16(cb, v);
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    H[k] = tc::f2_pack(__float_as_uint(v[2 * k]), __float_as_uint(v[2 * k + 1]));
                    L[k] = L2[k] = 0ull;
                }
#pragma unroll
                for (int d = 1; d <= D; d++) {
                    tc::tmem_ld16(cb + (uint32_t)(BN * d), v);
#pragma unroll
                    for (int k = 0; k < 8; k++) {
                        const uint64_t x =
                            tc::f2_pack(__float_as_uint(v[2 * k]), __float_as_uint(v[2 * k + 1]));
                        if (d == 1) {
                            const uint64_t hh = tc::f2_sub(tc::f2_add(x, C16), C16);
                            H[k] = tc::f2_add(H[k], hh);
                            L[k] = tc::f2_sub(x, hh);
                        } else if (d == 2) {
                            const uint64_t hh = tc::f2_sub(tc::f2_add(x, C25), C25);
                            L[k] = tc::f2_add(L[k], hh);
                            L2[k] = tc::f2_sub(x, hh);
                        } else {
                            L2[k] = tc::f2_add(L2[k], x);
                        }
                    }
                }
            }
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0)
                tc::mbar_arrive(tc::smem_u32(tempty));

            const int i = (t_begin + q) * Cfg::kPts + pt;  // r1 row of the tile
            if (i >= P.n1b)
                continue;
            // V_c 2^-ea = 2^eb_c ((H + L) + L2): TwoSum of H and L, then the rest.  The F
            // rows' scale 2^ea, a power of two common to the 16 values, multiplies the
            // results instead (the polynomial is linear in V, and power-of-two scaling
            // commutes with the double-float arithmetic).
            df::D V[16];
            const float *scr = Q.bscale + (int64_t)i * 16;  // 16-float aligned rows
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const uint64_t sm = tc::f2_add(H[k], L[k]);
                const uint64_t bb = tc::f2_sub(sm, H[k]);
                uint64_t e = tc::f2_add(tc::f2_sub(H[k], tc::f2_sub(sm, bb)), tc::f2_sub(L[k], bb));
                e = tc::f2_add(e, L2[k]);
                const uint64_t sc = *reinterpret_cast<const uint64_t *>(scr + 2 * k);
                const uint64_t hs = tc::f2_mul(sm, sc), ls = tc::f2_mul(e, sc);
                V[2 * k] = df::make(tc::f2_lo(hs), tc::f2_lo(ls));
                V[2 * k + 1] = df::make(tc::f2_hi(hs), tc::f2_hi(ls));
            }
            const int64_t o = (int64_t)i * P.ldg + j;
            float2 w4[4];
            if (jok) {
                const float2 *r1p = Q.r1d + 3 * (int64_t)i;
                const float2 r1x = r1p[0], r1y = r1p[1], r1z = r1p[2];
                df::D dx = df::sub(df::make(r1x.x, r1x.y), df::make(x2.x, x2.y));
                df::D dy = df::sub(df::make(r1y.x, r1y.y), df::make(y2.x, y2.y));
                df::D dz = df::sub(df::make(r1z.x, r1z.y), df::make(z2.x, z2.y));
                df::D d2 = df::add(df::add(df::sqr(dx), df::sqr(dy)), df::sqr(dz));
                bool coalesced = false;
                if (d2.hi < kNearPairR2) {
                    // near e-e coalescence the differences are taken in FP64, where they are
                    // exact (the coordinates' double-float forms keep only 48 bits); only g12
                    // and its gradient depend on them, so the rest stays as it is.  The
                    // reference's own guard, r12^2 <= 1e-15 (src/jast_bh.cu:143), gives g = 0.
                    const double *a1 = P.r1 + 3 * (int64_t)(P.i0 + i);
                    const double *a2 = P.r2 + 3 * (int64_t)j;
                    const double ex = a1[0] - a2[0], ey = a1[1] - a2[1], ez = a1[2] - a2[2];
                    dx = df::from_double(ex);
                    dy = df::from_double(ey);
                    dz = df::from_double(ez);
                    d2 = df::add(df::add(df::sqr(dx), df::sqr(dy)), df::sqr(dz));
                    coalesced = !(ex * ex + ey * ey + ez * ez > 1e-15);
                }
                df::D g = {0.f, 0.f}, gx = {0.f, 0.f}, gy = {0.f, 0.f}, gz = {0.f, 0.f};
                if (!coalesced) {
                    const df::D rd = df::sqrt(d2);
                    const df::D ar = df::mul(rd, a);
                    const df::D t = df::recip(df::add_f(ar, 1.0f));
                    g = df::mul(ar, t);
                    const df::D sg = df::mul(df::mul(df::sqr(t), a), df::recip(rd));
                    gx = df::mul(sg, dx);
                    gy = df::mul(sg, dy);
                    gz = df::mul(sg, dz);
                }
                const df::D g2 = df::sqr(g);
                // sum_o g^o V_o, o = 0, 2, 3, 4
                df::D ux = df::fma(df::fma(df::fma(V[3], g, V[2]), g, V[1]), g2, V[0]);
                df::D uy = df::fma(df::fma(df::fma(V[7], g, V[6]), g, V[5]), g2, V[4]);
                df::D uz = df::fma(df::fma(df::fma(V[11], g, V[10]), g, V[9]), g2, V[8]);
                const df::D dudg = df::mul(df::fma(df::fma(V[14], g, V[13]), g, V[12]), g);
                ux = df::fma(dudg, gx, ux);
                uy = df::fma(dudg, gy, uy);
                uz = df::fma(dudg, gz, uz);
                ux = df::make(__fmul_rn(ux.hi, sa), __fmul_rn(ux.lo, sa));
                uy = df::make(__fmul_rn(uy.hi, sa), __fmul_rn(uy.lo, sa));
                uz = df::make(__fmul_rn(uz.hi, sa), __fmul_rn(uz.lo, sa));
                const df::D n2v = df::add(df::add(df::sqr(ux), df::sqr(uy)), df::sqr(uz));
                const df::D lv = df::mul_f(n2v, -0.5f);
                w4[0] = make_float2(ux.hi, ux.lo);
                w4[1] = make_float2(uy.hi, uy.lo);
                w4[2] = make_float2(uz.hi, uz.lo);
                w4[3] = make_float2(lv.hi, lv.lo);
#pragma unroll
                for (int c = 0; c < 4; c++)
                    P.G[o + c * P.plane] = w4[c];
            }
            if (P.rmax) {
                // row maxima for the slicer from the float bits (as pair_df_kernel)
                const unsigned mask = __ballot_sync(0xffffffffu, jok);
                if (jok) {
                    const bool leader = lane == __ffs(mask) - 1;
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        const unsigned fb = __float_as_uint(w4[c].x) & 0x7fffffffu;
                        const unsigned m = rmax_word(__reduce_max_sync(mask, fb));
                        if (leader && m)
                            atomicMax(&P.rmax[(int64_t)c * P.n1b + i], (unsigned long long)m << 32);
                    }
                }
            }
        }
    }

    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == kCtlWarp)
        tc::tmem_dealloc(tbase, kTmemCols);
}

// ---------------------------------------------------------------------------
// slicing kernels
// ---------------------------------------------------------------------------

// Operand sources: value of row r, column k of an FP64 matrix.
struct SrcDense {  // X[r * ld + k]
    static constexpr bool kDoubleFloat = false;
    const double *X;
    int64_t ld;
    __device__ double operator()(int64_t r, int64_t k) const { return X[r * ld + k]; }
};

struct SrcConcat {  // [X1 | X2]: X1[r * k1 + k] for k < k1, then X2[r * k2 + k - k1]
    static constexpr bool kDoubleFloat = false;
    const double *X1, *X2;
    int64_t k1, k2;
    __device__ double operator()(int64_t r, int64_t k) const
    {
        return k < k1 ? X1[r * k1 + k] : X2[r * k2 + (k - k1)];
    }
};

struct SrcDenseDF {  // hi + lo of X[r * ld + k]; the slicer reads the pair itself
    static constexpr bool kDoubleFloat = true;
    const float2 *X;
    int64_t ld;
    __device__ float2 pair(int64_t r, int64_t k) const { return X[r * ld + k]; }
    __device__ double operator()(int64_t r, int64_t k) const
    {
        const float2 v = X[r * ld + k];
        return (double)v.x + (double)v.y;
    }
};

// The pair products take their first factor w chi_a from a table of the weighted AO
// rows, formed once per AO (weighted_aos_kernel) instead of once per pair: FP64
// multiplies run at 1/64 of the FP32 rate on GB300, and these sources are evaluated
// twice per element (row maxima, then digits).
struct SrcSym {  // w[k] chi_a(k) chi_b(k) = (w chi_a)(k) chi_b(k), (a, b) = pairs[r]
    static constexpr bool kDoubleFloat = false;
    const double *wchi, *chi;  // wchi[a * K + k] = w[k] chi_a(k); chi_b at chi[b * ldchi + k]
    int64_t K, ldchi;
    const int2 *pairs;
    __device__ double operator()(int64_t r, int64_t k) const
    {
        const int2 ab = pairs[r];
        return wchi[ab.x * K + k] * chi[ab.y * ldchi + k];
    }
};

// w (chi_c d_m chi_d - chi_d d_m chi_c) as (w chi_c) d_m chi_d - (w chi_d) d_m chi_c,
// k = m n + g, (c, d) = pairs[r]
struct SrcAnti {
    static constexpr bool kDoubleFloat = false;
    const double *wchi, *aos;  // wchi[c * n + g] = w[g] chi_c(g); aos: (ld, nA, 4) with
                               // the grid offset already applied
    int n, nA;                 // n: grid points counted in k (g < n)
    int64_t ld;                // grid stride of aos
    const int2 *pairs;
    __device__ double operator()(int64_t r, int64_t k) const
    {
        int m, g;
        if (k < 0x7fffffff) {  // 32-bit division (K = 3 n)
            const unsigned ku = (unsigned)k, mu = ku / (unsigned)n;
            m = (int)mu;
            g = (int)(ku - mu * (unsigned)n);
        } else {
            m = (int)(k / n);
            g = (int)(k % n);
        }
        const int2 cd = pairs[r];
        const int64_t comp = (int64_t)nA * ld * (m + 1);
        return fma(wchi[(int64_t)cd.x * n + g], aos[comp + cd.y * ld + g],
                   -(wchi[(int64_t)cd.y * n + g] * aos[comp + cd.x * ld + g]));
    }
};

// wchi[a * n + g] = w[g] chi_a(g), chi_a at chi[a * ldchi]
__global__ void weighted_aos_kernel(int n, const double *__restrict__ w,
                                    const double *__restrict__ chi, int64_t ldchi,
                                    double *__restrict__ wchi)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int a = blockIdx.y;
    if (g < n)
        wchi[(int64_t)a * n + g] = w[g] * chi[(int64_t)a * ldchi + g];
}

static int weighted_aos(cudaStream_t st, int n, int nA, const double *w, const double *chi,
                        int64_t ldchi, double *wchi)
{
    if (n <= 0 || nA <= 0)
        return CUTC_OK;
    weighted_aos_kernel<<<dim3(ceil_div(n, 256), nA), 256, 0, st>>>(n, w, chi, ldchi, wchi);
    CUTC_CUDA_TRY(cudaGetLastError());
    note_launches(1);
    return CUTC_OK;
}

// |v| as its bits (non-negative doubles order like their bits); NaN counts as 0, as
// fmax would skip it.  Integer work: an FP64 max would take the FP64 pipe.
__device__ __forceinline__ unsigned long long abs_bits(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    return b > 0x7ff0000000000000ull ? 0ull : b;
}

// rmax[r] = bits of max_k |src(r, k)|
template <class Src>
__global__ void rowmax_kernel(Src src, int rows, int64_t K, int64_t kper,
                              unsigned long long *rmax)
{
    const int r = blockIdx.x;
    if (r >= rows)
        return;
    const int64_t k0 = (int64_t)blockIdx.y * kper;
    const int64_t k1 = min(K, k0 + kper);
    unsigned long long m = 0;
    for (int64_t k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const unsigned long long b = abs_bits(src(r, k));
        m = b > m ? b : m;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long b = __shfl_xor_sync(0xffffffffu, m, o);
        m = b > m ? b : m;
    }
    __shared__ unsigned long long red[32];
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long b = __shfl_xor_sync(0xffffffffu, m, o);
            m = b > m ? b : m;
        }
        if (threadIdx.x == 0 && m > 0)
            atomicMax(&rmax[r], m);
    }
}

// Row maxima of a matrix stored column by column: src[(k0 + k) * ld + r].
__global__ void rowmax_cols_kernel(const double *X, int64_t ld, int64_t k0, int rows, int64_t K,
                                   int64_t kper, unsigned long long *rmax)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows)
        return;
    const int64_t ka = (int64_t)blockIdx.y * kper, kb = min(K, ka + kper);
    unsigned long long m = 0;
    for (int64_t k = ka; k < kb; k++) {
        const unsigned long long b = abs_bits(X[(k0 + k) * ld + r]);
        m = b > m ? b : m;
    }
    if (m > 0)
        atomicMax(&rmax[r], m);
}

// Exponent e with |x| < 2^e for every x of the row; 0 for zero (or denormal-only) rows.
__device__ __forceinline__ int row_exponent(unsigned long long bits)
{
    const int E = (int)((bits >> 52) & 0x7ff);
    return E == 0 ? 0 : E - 1022;
}

// The S signed base-2^9 digits of t (digits.cuh) as exact BF16 values q_s 2^{-8-9s}.
template <int S>
__device__ __forceinline__ void digits_of(long long t, __nv_bfloat16 (&out)[S])
{
    int q[S];
    digits::digits_int<S>(t, q);
#pragma unroll
    for (int s = 0; s < S; s++)
        out[s] = __float2bfloat16_rn(__int2float_rn(q[s]) * exp2f((float)(-8 - 9 * s)));
}

// The digits of an FP64 value x 2^{-e} (first digit scaled by 2^8).
template <int S>
__device__ __forceinline__ void split_digits(double x, int e, __nv_bfloat16 (&out)[S])
{
    digits_of<S>(digits::scaled_round<S>(x, e), out);
}

// slices[(s * Mpad + r) * Kpad + k] for r < Mpad, k < Kpad (zeros outside M x K);
// ex[r] = row exponent.  Four consecutive k per thread (Kpad is a multiple of 32),
// so each slice plane gets one 8-byte store per thread.  Rows are taken
// blockIdx.y, blockIdx.y + gridDim.y, ...: any row count fits the grid.
template <int S, class Src>
__global__ void slice_kernel(Src src, int M, int64_t K, int64_t Kpad, int Mpad,
                             const unsigned long long *rmax, __nv_bfloat16 *slices, int *ex)
{
    const int64_t k = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
    if (k >= Kpad)
        return;
    for (int r = blockIdx.y; r < Mpad; r += gridDim.y) {
        const int e = r < M ? row_exponent(rmax[r]) : 0;
        if (k == 0)
            ex[r] = e;
        __nv_bfloat16 d[4][S];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if constexpr (Src::kDoubleFloat) {
                const float2 v = (r < M && k + q < K) ? src.pair(r, k + q) : make_float2(0.f, 0.f);
                float qf[S];
                digits::digits_df_fp32<S>(v.x, v.y, e, qf);
#pragma unroll
                for (int s = 0; s < S; s++)
                    d[q][s] = __float2bfloat16_rn(__fmul_rn(qf[s], exp2f((float)(-8 - 9 * s))));
            } else {
                const double x = (r < M && k + q < K) ? src(r, k + q) : 0.0;
                split_digits<S>(x, e, d[q]);
            }
        }
#pragma unroll
        for (int s = 0; s < S; s++) {
            __nv_bfloat162 lo, hi;
            lo.x = d[0][s];
            lo.y = d[1][s];
            hi.x = d[2][s];
            hi.y = d[3][s];
            uint2 w;
            w.x = *reinterpret_cast<unsigned *>(&lo);
            w.y = *reinterpret_cast<unsigned *>(&hi);
            *reinterpret_cast<uint2 *>(slices + ((int64_t)s * Mpad + r) * Kpad + k) = w;
        }
    }
}

// Same for a matrix stored column by column, src[(k0 + k) * ld + r], through a
// 32 x 32 shared-memory transpose so reads and writes are both coalesced.
template <int S>
__global__ void slice_cols_kernel(const double *X, int64_t ld, int64_t k0, int M, int64_t K,
                                  int64_t Kpad, int Mpad, const unsigned long long *rmax,
                                  __nv_bfloat16 *slices, int *ex)
{
    __shared__ double tile[32][33];
    const int r0 = blockIdx.y * 32;
    const int64_t kb = (int64_t)blockIdx.x * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int i = ty; i < 32; i += blockDim.y) {
        const int64_t k = kb + i;
        const int r = r0 + tx;
        tile[i][tx] = (r < M && k < K) ? X[(k0 + k) * ld + r] : 0.0;
    }
    __syncthreads();
    for (int i = ty; i < 32; i += blockDim.y) {
        const int r = r0 + i;
        const int64_t k = kb + tx;
        if (r >= Mpad || k >= Kpad)
            continue;
        const int e = r < M ? row_exponent(rmax[r]) : 0;
        if (k == 0)
            ex[r] = e;
        __nv_bfloat16 d[S];
        split_digits<S>(tile[tx][i], e, d);
#pragma unroll
        for (int s = 0; s < S; s++)
            slices[((int64_t)s * Mpad + r) * Kpad + k] = d[s];
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

static inline int64_t round_up(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int get_encode(EncodeTiledFn *fn)
{
    static EncodeTiledFn cached = nullptr;
    if (!cached) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                         cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
            cudaGetLastError();
            cutc_set_error(CUTC_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
            return CUTC_ERR_CUDA;
        }
        cached = (EncodeTiledFn)p;
    }
    *fn = cached;
    return CUTC_OK;
}

// 2-D map over slices [rows_total][Kpad] BF16, box = kBK x box_rows, 64B swizzle.
static int make_tmap(CUtensorMap *map, const void *base, int64_t rows_total, int64_t Kpad,
                     int box_rows)
{
    EncodeTiledFn enc;
    CUTC_TRY(get_encode(&enc));
    cuuint64_t dims[2] = {(cuuint64_t)Kpad, (cuuint64_t)rows_total};
    cuuint64_t strides[1] = {(cuuint64_t)Kpad * 2};
    cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims,
                     strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        cutc_set_error(CUTC_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
        return CUTC_ERR_CUDA;
    }
    return CUTC_OK;
}


static int alloc_operand(Workspace &W, int slot, int S, int M, int row_mult, int64_t K,
                         Operand &op)
{
    op.M = M;
    op.Mpad = (int)round_up(std::max(M, 1), row_mult);
    op.K = K;
    op.Kpad = round_up(std::max<int64_t>(K, 1), kBK);
    void *p;
    CUTC_TRY(W.get(slot, (size_t)S * op.Mpad * op.Kpad * 2, &p));
    op.sl = p;
    CUTC_TRY(W.get(slot + 1, (size_t)op.Mpad * 4, &p));
    op.ex = (int *)p;
    CUTC_TRY(W.get(slot + 2, (size_t)op.Mpad * 8, &p));
    op.rmax = (unsigned long long *)p;
    return CUTC_OK;
}

// have_rmax: op.rmax already holds the row maxima (written by the producer of src)
template <int S, class Src>
static int slice_rows(cudaStream_t st, Src src, Operand &op, bool have_rmax = false)
{
    if (!have_rmax) {
        CUTC_CUDA_TRY(cudaMemsetAsync(op.rmax, 0, (size_t)op.Mpad * 8, st));
        if (op.M > 0 && op.K > 0) {
            const int64_t kper = 16384;
            dim3 g1((unsigned)op.M, ceil_div(op.K, kper));
            rowmax_kernel<Src><<<g1, 256, 0, st>>>(src, op.M, op.K, kper, op.rmax);
            CUTC_CUDA_TRY(cudaGetLastError());
        }
    }
    if (op.Kpad % 4) {
        cutc_set_error(CUTC_ERR_INVALID, "operand K padding %lld is not a multiple of 4",
                       (long long)op.Kpad);
        return CUTC_ERR_INVALID;
    }
    dim3 g2(ceil_div(op.Kpad, 4 * 256), (unsigned)std::min(op.Mpad, 65535));
    slice_kernel<S, Src><<<g2, 256, 0, st>>>(src, op.M, op.K, op.Kpad, op.Mpad, op.rmax,
                                             (__nv_bfloat16 *)op.sl, op.ex);
    CUTC_CUDA_TRY(cudaGetLastError());
    note_launches(have_rmax ? 1 : 2);
    return CUTC_OK;
}

template <int S>
static int slice_cols(cudaStream_t st, const double *X, int64_t ld, int64_t k0, Operand &op)
{
    CUTC_CUDA_TRY(cudaMemsetAsync(op.rmax, 0, (size_t)op.Mpad * 8, st));
    if (op.M > 0 && op.K > 0) {
        const int64_t kper = 512;
        dim3 g1(ceil_div(op.M, 128), ceil_div(op.K, kper));
        rowmax_cols_kernel<<<g1, 128, 0, st>>>(X, ld, k0, op.M, op.K, kper, op.rmax);
        CUTC_CUDA_TRY(cudaGetLastError());
    }
    dim3 g2(ceil_div(op.Kpad, 32), ceil_div(op.Mpad, 32));
    slice_cols_kernel<S><<<g2, dim3(32, 8), 0, st>>>(X, ld, k0, op.M, op.K, op.Kpad, op.Mpad,
                                                     op.rmax, (__nv_bfloat16 *)op.sl, op.ex);
    CUTC_CUDA_TRY(cudaGetLastError());
    note_launches(2);
    return CUTC_OK;
}

int split_k_blocks_per_launch(int64_t K, int64_t M, int k_split)
{
    const int64_t nkb_total = (std::max<int64_t>(K, 1) + kBK - 1) / kBK;
    if (k_split > 0)
        return std::max(1, std::min(k_split, kMaxKPerLaunch) / kBK);
    const int64_t kt = nkb_total * kBK;
    const bool big = M >= kBigM;
    const int64_t one = big ? kLongKBigM : kLongK, each = big ? kLaunchKBigM : kLaunchK;
    const int64_t launches = kt <= one ? 1 : (kt + each - 1) / each;
    return (int)((nkb_total + launches - 1) / launches);
}

// C = alpha A B^T (+ C) over the operands' common K.
template <int S>
static int gemm(cudaStream_t st, const Operand &A, const Operand &B, double alpha, double *C,
                int64_t ldc, int ncol_group, int64_t group_stride, int64_t col0, int accumulate,
                int *err, int k_split = 0)
{
    using Cfg = GemmCfg<S>;
    static std::atomic<unsigned long long> attr_done{0};
    const unsigned long long bit = current_device_bit();
    if (!(attr_done.load() & bit)) {
        CUTC_CUDA_TRY(cudaFuncSetAttribute(split_gemm_kernel<S>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmem));
        attr_done.fetch_or(bit);
    }
    CUtensorMap ta, tb;
    CUTC_TRY(make_tmap(&ta, A.sl, (int64_t)S * A.Mpad, A.Kpad, kBM));
    CUTC_TRY(make_tmap(&tb, B.sl, (int64_t)S * B.Mpad, B.Kpad, Cfg::kBN));
    const int nkb_total = (int)(A.Kpad / kBK);
    const int kb_per = split_k_blocks_per_launch(A.Kpad, A.M, k_split);
    if (A.Mpad % kBM || B.Mpad % Cfg::kBN) {
        cutc_set_error(CUTC_ERR_INVALID, "operand padding does not match the tile");
        return CUTC_ERR_INVALID;
    }
    dim3 grid((unsigned)((int64_t)(A.Mpad / kBM) * (B.Mpad / Cfg::kBN)));
    for (int kb0 = 0; kb0 < nkb_total; kb0 += kb_per) {
        GemmParams P;
        P.M = A.M;
        P.N = B.M;
        P.Mpad = A.Mpad;
        P.Npad = B.Mpad;
        P.kb0 = kb0;
        P.nkb = std::min(kb_per, nkb_total - kb0);
        P.ea = A.ex;
        P.eb = B.ex;
        // a power of two (1, -1/2, 1/2 in this library) scales through the exponent
        int ae = 0;
        const double am = std::frexp(std::fabs(alpha), &ae);
        P.alpha_mul = am != 0.5;
        P.alpha_exp = P.alpha_mul ? 0 : ae - 1;
        P.alpha_neg = !P.alpha_mul && alpha < 0;
        P.alpha = alpha;
        P.C = C;
        P.ldc = ldc;
        P.ncol_group = ncol_group;
        P.group_stride = group_stride;
        P.col0 = col0;
        P.accumulate = (accumulate || kb0 > 0) ? 1 : 0;
        P.err = err;
        split_gemm_kernel<S><<<grid, Cfg::kThreads, Cfg::kSmem, st>>>(ta, tb, P);
        CUTC_CUDA_TRY(cudaGetLastError());
        note_launches(1);
    }
    return CUTC_OK;
}

// ---------------------------------------------------------------------------
// the plan for one build
// ---------------------------------------------------------------------------

enum SplitSlot {
    SS_PAIRS_SYM = 0, SS_PAIRS_ANTI = 1, SS_ERR = 2,
    SS_AX = 3, SS_BX = 6, SS_AH = 9, SS_AN = 12, SS_BH = 15, SS_BN = 18,
    SS_AF = 21, SS_BC = 24, SS_F64 = 27, SS_C64 = 28, SS_R1D = 29, SS_BSCALE = 30,
    SS_WCHI2 = 31, SS_WCHI1 = 32,
};


size_t split_r1_row_bytes(const Request &R)
{
    // slices of the four G rows of one r1 point
    return 2 * (size_t)R.n_slices * 4 * (size_t)round_up(R.n2, kBK) + 64;
}

size_t split_int2e_row_bytes(const Request &R)
{
    const int64_t np = n_pairs(R.nA), nl = std::max<int64_t>(1, n_strict_pairs(R.nA));
    const int bn = bn_for(R.n_slices);
    // the point's K columns of the int_2e operands (X_3, X_012, S0, S), and its
    // weighted AO values w chi_a
    return 2 * (size_t)R.n_slices * (round_up(np, kBM) * 4 + round_up(np, bn) +
                                     3 * (size_t)round_up(nl, bn)) + 8 * (size_t)R.nA + 64;
}

size_t split_fixed_bytes(const Request &R)
{
    // P slices and the weighted AO values w chi_a on r2 they are formed from
    return 2 * (size_t)R.n_slices * round_up(n_pairs(R.nA), kBM) * round_up(R.n2, kBK) +
           8 * (size_t)R.nA * R.n2;
}

static int upload_pairs(Workspace &W, int slot, cudaStream_t st, int nA, bool strict, int2 **out)
{
    std::vector<int2> v;
    for (int b = 0; b < nA; b++)
        for (int a = strict ? b + 1 : b; a < nA; a++)
            v.push_back(make_int2(a, b));  // packed order of tri_index / stri_index
    void *p;
    CUTC_TRY(W.get(slot, std::max<size_t>(1, v.size()) * sizeof(int2), &p));
    if (!v.empty())
        CUTC_CUDA_TRY(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
    CUTC_CUDA_TRY(cudaStreamSynchronize(st));  // v goes out of scope
    *out = (int2 *)p;
    return CUTC_OK;
}

#define CUTC_SLICES_DISPATCH(S_, CALL)                                         \
    switch (S_) {                                                              \
    case 3: { constexpr int S = 3; CALL; } break;                              \
    case 4: { constexpr int S = 4; CALL; } break;                              \
    case 5: { constexpr int S = 5; CALL; } break;                              \
    case 6: { constexpr int S = 6; CALL; } break;                              \
    case 7: { constexpr int S = 7; CALL; } break;                              \
    default:                                                                   \
        cutc_set_error(CUTC_ERR_INVALID, "unsupported slice count %d", S_);    \
        return CUTC_ERR_INVALID;                                               \
    }

int split_prepare_x(Engine *E, const Request &R, cudaStream_t st, const double *wr2,
                    const double *aos2v, int64_t n1t, int slot0, SplitPlan &sp)
{
    Workspace &W = E->ws;
    SplitPlan &S_ = sp;
    sp.slot0 = slot0;
    sp.n_slices = R.n_slices;
    sp.n1t = n1t;
    const int np = (int)n_pairs(R.nA);
    void *p;
    CUTC_TRY(W.get(slot0 + SS_ERR, 64, &p));
    S_.err = (int *)p;
    CUTC_CUDA_TRY(cudaMemsetAsync(S_.err, 0, 4, st));
    CUTC_TRY(upload_pairs(W, slot0 + SS_PAIRS_SYM, st, R.nA, false, &S_.pairs_sym));
    CUTC_TRY(upload_pairs(W, slot0 + SS_PAIRS_ANTI, st, R.nA, true, &S_.pairs_anti));
    CUTC_TRY(alloc_operand(W, slot0 + SS_AX, R.n_slices, np, kBM, R.n2, S_.AX));
    CUTC_TRY(alloc_operand(W, slot0 + SS_BX, R.n_slices, (int)(4 * n1t), bn_for(R.n_slices), R.n2,
                           S_.BX));
    if (R.mol_tag && E->tag_x == R.mol_tag && E->tag_x_buf == S_.AX.sl)
        return CUTC_OK;  // the same molecule's P slices are already there
    CUTC_TRY(W.get(slot0 + SS_WCHI2, std::max<size_t>(1, (size_t)R.nA * R.n2) * 8, &p));
    double *wchi = (double *)p;
    CUTC_TRY(weighted_aos(st, R.n2, R.nA, wr2, aos2v, (int64_t)R.n2, wchi));
    SrcSym src{wchi, aos2v, (int64_t)R.n2, (int64_t)R.n2, S_.pairs_sym};
    CUTC_SLICES_DISPATCH(R.n_slices, CUTC_TRY((slice_rows<S, SrcSym>(st, src, S_.AX))));
    E->tag_x = R.mol_tag;
    E->tag_x_buf = S_.AX.sl;
    return CUTC_OK;
}

int split_x_tile(Engine *E, const Request &R, cudaStream_t st, SplitPlan &sp, const float2 *G,
                 int nb, double *Xb, int blk_rows, int ib, cudaEvent_t gemm_begin,
                 cudaEvent_t gemm_end, bool have_rmax)
{
    (void)E;
    SplitPlan &S_ = sp;
    Operand B = S_.BX;
    B.M = 4 * nb;  // rows (c, i) of this tile; Mpad keeps the allocated padding
    B.Mpad = (int)round_up(B.M, bn_for(sp.n_slices));
    const int64_t np = n_pairs(R.nA);
    SrcDenseDF src{G, (int64_t)R.n2};
    CUTC_SLICES_DISPATCH(sp.n_slices, {
        CUTC_TRY((slice_rows<S, SrcDenseDF>(st, src, B, have_rmax)));
        if (gemm_begin)
            CUTC_CUDA_TRY(cudaEventRecord(gemm_begin, st));
        // column (c, i) of the tile -> column c blk_rows + ib + i of the block
        CUTC_TRY((gemm<S>(st, S_.AX, B, 1.0, Xb, np, nb, blk_rows, ib, 0, S_.err, R.k_split)));
        if (gemm_end)
            CUTC_CUDA_TRY(cudaEventRecord(gemm_end, st));
    });
    return CUTC_OK;
}

int split_int2e_tile(Engine *E, const Request &R, cudaStream_t st, SplitPlan &sp,
                     const double *wr1, const double *aos1, int64_t ld1, int nb, const double *Xt,
                     double *H, double *N, bool first)
{
    Workspace &W = E->ws;
    SplitPlan &S_ = sp;
    const int slot0 = sp.slot0;
    const int nA = R.nA;
    const int np = (int)n_pairs(nA), nl = (int)n_strict_pairs(nA);
    const int bn = bn_for(sp.n_slices);
    Operand AH, AN, BH, BN;
    CUTC_TRY(alloc_operand(W, slot0 + SS_AH, sp.n_slices, np, kBM, nb, AH));
    CUTC_TRY(alloc_operand(W, slot0 + SS_AN, sp.n_slices, np, kBM, 3 * (int64_t)nb, AN));
    CUTC_TRY(alloc_operand(W, slot0 + SS_BH, sp.n_slices, np, bn, nb, BH));
    CUTC_TRY(alloc_operand(W, slot0 + SS_BN, sp.n_slices, std::max(nl, 1), bn, 3 * (int64_t)nb, BN));
    BN.M = nl;
    const int acc = first ? 0 : 1;
    // With the whole r1 grid in one tile the B operands depend on the molecule
    // only, and a build with the same molecule tag keeps them.
    const bool keep_b = nb == R.n1 && R.mol_tag && E->tag_i == R.mol_tag && E->tag_i_buf == BH.sl;
    void *p;
    CUTC_TRY(W.get(slot0 + SS_WCHI1, std::max<size_t>(1, (size_t)nA * nb) * 8, &p));
    double *wchi = (double *)p;
    if (!keep_b)
        CUTC_TRY(weighted_aos(st, nb, nA, wr1, aos1, ld1, wchi));
    SrcSym s0{wchi, aos1, (int64_t)nb, ld1, S_.pairs_sym};
    SrcAnti sa{wchi, aos1, nb, nA, ld1, S_.pairs_anti};
    CUTC_SLICES_DISPATCH(sp.n_slices, {
        // Xt[(m nb + i) np + p]: X_3 is column block 3, X_012 the blocks 0..2
        CUTC_TRY(slice_cols<S>(st, Xt, np, 3 * (int64_t)nb, AH));
        CUTC_TRY(slice_cols<S>(st, Xt, np, 0, AN));
        if (!keep_b) {
            CUTC_TRY((slice_rows<S, SrcSym>(st, s0, BH)));
            if (nl > 0)
                CUTC_TRY((slice_rows<S, SrcAnti>(st, sa, BN)));
        }
        CUTC_TRY(gemm<S>(st, AH, BH, 1.0, H, np, np, 0, 0, acc, S_.err, R.k_split));
        if (nl > 0)
            CUTC_TRY(gemm<S>(st, AN, BN, -0.5, N, np, nl, 0, 0, acc, S_.err, R.k_split));
    });
    if (nb == R.n1) {
        E->tag_i = R.mol_tag;
        E->tag_i_buf = BH.sl;
    } else {
        E->tag_i = 0;
    }
    return CUTC_OK;
}

// ---- pair terms on the tensor cores -------------------------------------------------

constexpr int kPairTcMaxNuc = 20;  // K = 4 n_nuc <= 80 keeps diagonals 0..2 exact

// Slices of the pair contraction's operands: 5 (representation error 2^-45, under the
// error of a 5-slice build's contractions), or 6 for builds of 6 and 7 slices, whose
// contractions reach FP64-class errors (2^-54, below the double-float epilogue).
static int pair_tc_slices(const Request &R) { return R.n_slices >= 6 ? 6 : 5; }

bool split_pair_tc_ok(const Request &R, const int *exps, int n_terms)
{
    return R.precision == CUTC_SPLIT_BF16 && !R.pair_fp64 && R.nN <= kPairTcMaxNuc &&
           pair_df_sparse(exps, n_terms) && !getenv("CUTC_PAIR_DF") && !getenv("CUTC_PAIR_DENSE");
}

size_t split_pair_fixed_bytes(const Request &R)
{
    const int64_t K = 4 * (int64_t)R.nN;
    return (size_t)R.n2 * K * 8 +
           2 * (size_t)pair_tc_slices(R) * round_up(R.n2, kBM) * round_up(K, kBK);
}

size_t split_pair_row_bytes(const Request &R)
{
    const int64_t K = 4 * (int64_t)R.nN;
    return 16 * (size_t)K * 8 + 2 * (size_t)pair_tc_slices(R) * 16 * round_up(K, kBK) + 3 * 8 +
           16 * 4 + 64;
}

int split_pair_prepare(Engine *E, const Request &R, cudaStream_t st, const double *f2,
                       int64_t n1t, SplitPlan &sp)
{
    Workspace &W = E->ws;
    const int slot0 = sp.slot0;
    const int64_t K = 4 * (int64_t)R.nN;
    void *p;
    CUTC_TRY(W.get(slot0 + SS_F64, (size_t)R.n2 * K * 8, &p));
    sp.Fd = (double *)p;
    CUTC_TRY(W.get(slot0 + SS_C64, (size_t)16 * n1t * K * 8, &p));
    sp.Cd = (double *)p;
    CUTC_TRY(W.get(slot0 + SS_R1D, (size_t)3 * n1t * sizeof(float2), &p));
    sp.r1d = (float2 *)p;
    CUTC_TRY(W.get(slot0 + SS_BSCALE, (size_t)round_up(16 * n1t, kPairBN) * 4, &p));
    sp.bscale = (float *)p;
    const int ps = pair_tc_slices(R);
    CUTC_TRY(alloc_operand(W, slot0 + SS_AF, ps, R.n2, kBM, K, sp.AF));
    CUTC_TRY(alloc_operand(W, slot0 + SS_BC, ps, (int)(16 * n1t), kPairBN, K, sp.BC));
    CUTC_TRY(launch_pair_tc_f(st, R.n2, R.nN, f2, sp.Fd));
    note_launches(1);
    SrcDense src{sp.Fd, K};
    if (ps == 6)
        CUTC_TRY((slice_rows<6, SrcDense>(st, src, sp.AF)));
    else
        CUTC_TRY((slice_rows<5, SrcDense>(st, src, sp.AF)));
    sp.pair_slices = ps;
    sp.pair_tc = true;
    return CUTC_OK;
}

template <int S, int KB>
static int launch_pair_tc_kernel(cudaStream_t st, const CUtensorMap &ta, const CUtensorMap &tb,
                                 PairTcParams Q, int n_sm)
{
    using Cfg = PairTcCfg<S, KB>;
    static std::atomic<unsigned long long> attr_done{0};
    const unsigned long long bit = current_device_bit();
    if (!(attr_done.load() & bit)) {
        CUTC_CUDA_TRY(cudaFuncSetAttribute(pair_tc_kernel<S, KB>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmem));
        attr_done.fetch_or(bit);
    }
    // about eight CTAs per SM, each walking a run of N tiles with its F tile resident
    const int64_t want = 8 * (int64_t)n_sm;
    const int64_t chunks = std::max<int64_t>(
        1, std::min<int64_t>(Q.tiles_n, (want + Q.tiles_m - 1) / Q.tiles_m));
    Q.chunk = (int)((Q.tiles_n + chunks - 1) / chunks);
    const int64_t grid = (int64_t)Q.tiles_m * ((Q.tiles_n + Q.chunk - 1) / Q.chunk);
    if (grid > INT32_MAX) {
        cutc_set_error(CUTC_ERR_INVALID, "pair grid of %lld CTAs", (long long)grid);
        return CUTC_ERR_INVALID;
    }
    pair_tc_kernel<S, KB><<<(unsigned)grid, Cfg::kThreads, Cfg::kSmem, st>>>(ta, tb, Q);
    CUTC_CUDA_TRY(cudaGetLastError());
    return CUTC_OK;
}

template <int S>
static int pair_tile(Engine *E, cudaStream_t st, SplitPlan &sp, const PairDfArgs &P,
                     const double *rn, double a_en)
{
    constexpr int BN = kPairBN;
    const int64_t K = 4 * (int64_t)P.nN;
    CUTC_TRY(launch_pair_tc_coef(st, P.i0, P.n1b, P.nN, P.r1, rn, a_en, P.coef, P.exps,
                                 P.term_off, sp.Cd, sp.r1d));
    Operand B = sp.BC;
    B.M = 16 * P.n1b;
    B.Mpad = (int)round_up(B.M, BN);
    SrcDense src{sp.Cd, K};
    CUTC_TRY((slice_rows<S, SrcDense>(st, src, B)));
    exp_scale_kernel<<<ceil_div(B.Mpad, 256), 256, 0, st>>>(B.ex, B.Mpad, sp.bscale);
    CUTC_CUDA_TRY(cudaGetLastError());
    CUtensorMap ta, tb;
    CUTC_TRY(make_tmap(&ta, sp.AF.sl, (int64_t)S * sp.AF.Mpad, sp.AF.Kpad, kBM));
    CUTC_TRY(make_tmap(&tb, B.sl, (int64_t)S * B.Mpad, B.Kpad, BN));
    PairTcParams Q;
    Q.tiles_m = sp.AF.Mpad / kBM;
    Q.tiles_n = B.Mpad / BN;
    Q.chunk = 1;
    Q.Mpad = sp.AF.Mpad;
    Q.Npad = B.Mpad;
    Q.ea = sp.AF.ex;
    Q.bscale = sp.bscale;
    Q.r1d = sp.r1d;
    Q.P = P;
    Q.err = sp.err;
    const int KB = (int)(sp.AF.Kpad / kBK);
    switch (KB) {
    case 1: CUTC_TRY((launch_pair_tc_kernel<S, 1>(st, ta, tb, Q, E->n_sm))); break;
    case 2: CUTC_TRY((launch_pair_tc_kernel<S, 2>(st, ta, tb, Q, E->n_sm))); break;
    case 3: CUTC_TRY((launch_pair_tc_kernel<S, 3>(st, ta, tb, Q, E->n_sm))); break;
    default:
        cutc_set_error(CUTC_ERR_INVALID, "pair contraction of K = %lld", (long long)K);
        return CUTC_ERR_INVALID;
    }
    note_launches(3);
    return CUTC_OK;
}

int split_pair_tile(Engine *E, const Request &R, cudaStream_t st, SplitPlan &sp,
                    const PairDfArgs &P, const double *rn, double a_en)
{
    (void)R;
    if (P.n1b <= 0 || P.n2 <= 0)
        return CUTC_OK;
    return sp.pair_slices == 6 ? pair_tile<6>(E, st, sp, P, rn, a_en)
                               : pair_tile<5>(E, st, sp, P, rn, a_en);
}

// One CTA waits on a pipeline barrier that nothing completes, with the bounded wait
// the tensor-core kernels use; it records whether the wait gave up (2) or, against
// all expectation, completed (1).
__global__ void wait_limit_kernel(int *result)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        tc::mbar_init(tc::smem_u32(&bar), 1);
        tc::fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0)
        *result = tc::mbar_wait(tc::smem_u32(&bar), 0, nullptr) ? 1 : 2;
}

int split_wait_limit_check(Engine *E)
{
    void *p;
    CUTC_TRY(E->ws.get(240, 64, &p));
    int *d = (int *)p;
    CUTC_CUDA_TRY(cudaMemsetAsync(d, 0, 4, E->stream));
    wait_limit_kernel<<<1, 32, 0, E->stream>>>(d);
    CUTC_CUDA_TRY(cudaGetLastError());
    int h = 0;
    CUTC_CUDA_TRY(cudaMemcpyAsync(&h, d, 4, cudaMemcpyDeviceToHost, E->stream));
    CUTC_CUDA_TRY(cudaStreamSynchronize(E->stream));
    if (h == 2) {
        cutc_set_error(CUTC_ERR_TIMEOUT, "a pipeline wait gave up after its limit (as checked)");
        return CUTC_ERR_TIMEOUT;
    }
    cutc_set_error(CUTC_ERR_CUDA, "the wait-limit check's barrier completed (result %d)", h);
    return CUTC_ERR_CUDA;
}

int split_check(cudaStream_t st, SplitPlan &sp)
{
    int herr = 0;
    CUTC_CUDA_TRY(cudaMemcpyAsync(&herr, sp.err, 4, cudaMemcpyDeviceToHost, st));
    CUTC_CUDA_TRY(cudaStreamSynchronize(st));
    if (herr) {
        cutc_set_error(CUTC_ERR_TIMEOUT, "a tensor-core pipeline wait gave up (code %d)", herr);
        return CUTC_ERR_TIMEOUT;
    }
    return CUTC_OK;
}

// Split-precision GEMM on device arrays: C[m + ldc n] = sum_k A[m K + k] B[n K + k].
int split_gemm_dense(Engine *E, cudaStream_t st, int n_slices, int M, int N, int64_t K,
                     const double *A, const double *B, double *C, int64_t ldc)
{
    Workspace &W = E->ws;
    const int base = 200;
    Operand OA, OB;
    CUTC_TRY(alloc_operand(W, base, n_slices, M, kBM, K, OA));
    CUTC_TRY(alloc_operand(W, base + 3, n_slices, N, bn_for(n_slices), K, OB));
    void *p;
    CUTC_TRY(W.get(base + 6, 64, &p));
    int *err = (int *)p;
    CUTC_CUDA_TRY(cudaMemsetAsync(err, 0, 4, st));
    SrcDense sa{A, K}, sb{B, K};
    CUTC_SLICES_DISPATCH(n_slices, {
        CUTC_TRY((slice_rows<S, SrcDense>(st, sa, OA)));
        CUTC_TRY((slice_rows<S, SrcDense>(st, sb, OB)));
        CUTC_TRY(gemm<S>(st, OA, OB, 1.0, C, ldc, N, 0, 0, 0, err));
    });
    int herr = 0;
    CUTC_CUDA_TRY(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
    CUTC_CUDA_TRY(cudaStreamSynchronize(st));
    if (herr) {
        cutc_set_error(CUTC_ERR_TIMEOUT, "a tensor-core pipeline wait gave up (code %d)", herr);
        return CUTC_ERR_TIMEOUT;
    }
    return CUTC_OK;
}

// C[m + ldc n] = alpha sum_k [A1 | A2][m, k] [B1 | B2][n, k] through the split form: the
// two products of the same output as ONE contraction over K1 + K2 (one row scale per row
// of the concatenation, exact accumulation over all of it).  A1, B1 are K1-contiguous,
// A2, B2 K2-contiguous (device arrays); synchronous on st.
int split_gemm_concat(Engine *E, cudaStream_t st, int n_slices, int M, int N, int64_t K1,
                      const double *A1, const double *B1, int64_t K2, const double *A2,
                      const double *B2, double alpha, double *C, int64_t ldc)
{
    Workspace &W = E->ws;
    const int base = 210;
    const int64_t K = K1 + K2;
    Operand OA, OB;
    CUTC_TRY(alloc_operand(W, base, n_slices, M, kBM, K, OA));
    CUTC_TRY(alloc_operand(W, base + 3, n_slices, N, bn_for(n_slices), K, OB));
    void *p;
    CUTC_TRY(W.get(base + 6, 64, &p));
    int *err = (int *)p;
    CUTC_CUDA_TRY(cudaMemsetAsync(err, 0, 4, st));
    SrcConcat sa{A1, A2, K1, K2}, sb{B1, B2, K1, K2};
    CUTC_SLICES_DISPATCH(n_slices, {
        CUTC_TRY((slice_rows<S, SrcConcat>(st, sa, OA)));
        CUTC_TRY((slice_rows<S, SrcConcat>(st, sb, OB)));
        CUTC_TRY(gemm<S>(st, OA, OB, alpha, C, ldc, N, 0, 0, 0, err));
    });
    int herr = 0;
    CUTC_CUDA_TRY(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
    CUTC_CUDA_TRY(cudaStreamSynchronize(st));
    if (herr) {
        cutc_set_error(CUTC_ERR_TIMEOUT, "a tensor-core pipeline wait gave up (code %d)", herr);
        return CUTC_ERR_TIMEOUT;
    }
    return CUTC_OK;
}

}  // namespace cutc
