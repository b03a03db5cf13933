// Pair terms grad1 u(r1, r2) in double-float arithmetic (split form, sm_103a).
//
// Same quantity as pair.cu (the reference's cutc_int_bh_kernel,
// src/jast_bh.cu:31-264), reorganised so that the O(n1 n2) part runs on the
// FP32 pipes, which issue 64x faster than FP64 on GB300:
//
//   For nucleus A the Jastrow terms give two polynomials in (f2A, g12),
//     du/df1A = sum_{b,o} U_A[b][o](r1) f2A^b g^o
//     du/dg   = sum_A sum_{b,o'} W_A[b][o'](r1) f2A^b g^o'
//   with the r1-dependent coefficients
//     U[n][o] += c m f1^{m-1},  U[m][o] += c n f1^{n-1}
//     W[n][o-1] += c o f1^m,    W[m][o-1] += c o f1^n       (term (c, m, n, o))
//   computed once per (r1, nucleus) in FP64 by r1_poly_kernel.  Per pair the
//   kernel evaluates both polynomials by Horner's rule in df arithmetic
//   (~43 df multiply-adds per nucleus for exponents <= 4), then
//     grad1 u = sum_A du/df1A grad f1A + du/dg grad g12.
//   * For pairs closer than 0.01 bohr (e-e coalescence) the coordinate
//     differences are taken in FP64, where they are exact, and the reference's
//     r^2 > 1e-15 guard applies; e-n coalescence is handled by the FP64
//     per-point terms.
//   * Output is G[c][i][j] as (hi, lo) float pairs; hi + lo is exact in FP64.
#include <algorithm>

#include "common.cuh"
#include "dfloat.cuh"
#include "pair.cuh"

namespace cutc {

constexpr int kDfThreads = 128;

template <int E>
struct PolyLayout {
    static constexpr int kU = (E + 1) * (E + 1);  // U[b][o]
    static constexpr int kW = (E + 1) * E;        // W[b][o'], o' = o - 1
    static constexpr int kN = kU + kW + 3;        // + grad f1 (x, y, z)
};

// coef[(i * nN + A) * kN + ...] for rows i of the tile, in df
template <int E>
__global__ void r1_poly_kernel(int i0, int n, int nN, const double *__restrict__ r1,
                               const double *__restrict__ rn, double a_en,
                               const double *__restrict__ tcoef, const int *__restrict__ texps,
                               const int *__restrict__ toff, float2 *__restrict__ out)
{
    using L = PolyLayout<E>;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * nN)
        return;
    const int i = (int)(idx / nN), A = (int)(idx % nN);
    const double *p = r1 + 3 * (int64_t)(i0 + i);
    const double dx = p[0] - rn[3 * A], dy = p[1] - rn[3 * A + 1], dz = p[2] - rn[3 * A + 2];
    const double d2 = dx * dx + dy * dy + dz * dz;
    double f = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
    if (d2 > 1e-15) {
        const double d = sqrt(d2);
        const double t = 1.0 / (1.0 + a_en * d);
        f = a_en * d * t;
        const double s = a_en * t * t / d;
        gx = s * dx;
        gy = s * dy;
        gz = s * dz;
    }
    double F[kMaxExp + 1];
    F[0] = 1.0;
    for (int k = 1; k <= kMaxExp; k++)
        F[k] = F[k - 1] * f;
    double U[L::kU], W[L::kW];
    for (int k = 0; k < L::kU; k++)
        U[k] = 0.0;
    for (int k = 0; k < L::kW; k++)
        W[k] = 0.0;
    for (int k = toff[A]; k < toff[A + 1]; k++) {
        const int e = texps[k];
        const int m = e & 7, nn = (e >> 3) & 7, o = (e >> 6) & 7;
        const double cm = tcoef[3 * k], cn = tcoef[3 * k + 1], co = tcoef[3 * k + 2];
        if (m > 0)
            U[nn * (E + 1) + o] += cm * F[m - 1];
        if (nn > 0)
            U[m * (E + 1) + o] += cn * F[nn - 1];
        if (o > 0) {
            W[nn * E + o - 1] += co * F[m];
            W[m * E + o - 1] += co * F[nn];
        }
    }
    float2 *dst = out + idx * L::kN;
    for (int k = 0; k < L::kU; k++) {
        const df::D v = df::from_double(U[k]);
        dst[k] = make_float2(v.hi, v.lo);
    }
    for (int k = 0; k < L::kW; k++) {
        const df::D v = df::from_double(W[k]);
        dst[L::kU + k] = make_float2(v.hi, v.lo);
    }
    const double gg[3] = {gx, gy, gz};
    for (int c = 0; c < 3; c++) {
        const df::D v = df::from_double(gg[c]);
        dst[L::kU + L::kW + c] = make_float2(v.hi, v.lo);
    }
}

// r2 coordinates and f2A in df: r2d[c * n2 + j], f2d[A * n2 + j]
__global__ void r2_df_kernel(int n2, int nN, const double *__restrict__ r2,
                             const double *__restrict__ f2, float2 *__restrict__ r2d,
                             float2 *__restrict__ f2d)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n2)
        return;
    for (int c = 0; c < 3; c++) {
        const df::D v = df::from_double(r2[3 * (int64_t)j + c]);
        r2d[(int64_t)c * n2 + j] = make_float2(v.hi, v.lo);
    }
    for (int A = 0; A < nN; A++) {
        const df::D v = df::from_double(f2[(int64_t)A * n2 + j]);
        f2d[(int64_t)A * n2 + j] = make_float2(v.hi, v.lo);
    }
}

// Sp: every Jastrow exponent is 0, 2, 3 or 4 (E == 4).  Then U[b][o] and W[b][o'] vanish
// for b = 1, o = 1 and o' = 0, and the polynomials are evaluated as
//   sum_{b in 0,2,3,4} f2^b p_b(g) = p_0 + f2^2 (p_2 + f2 (p_3 + f2 p_4)),
//   p_b(g) = U[b][0] + g^2 (U[b][2] + g (U[b][3] + g U[b][4])),
// with g^2 per pair and f2^2 per nucleus, and the W part with its common factor g
// taken out of the nucleus sum: 30 df multiply-adds per nucleus instead of 46.
template <int E, bool Sp>
__global__ void __launch_bounds__(kDfThreads)
pair_df_kernel(PairDfArgs P)
{
    static_assert(!Sp || E == 4, "the sparse-power form is for exponents up to 4");
    using L = PolyLayout<E>;
    extern __shared__ __align__(16) float2 s_coef[];  // [row][A][kN], then r1 df [row][3]
    const int rows = P.rows_per_cta;
    const int row0 = blockIdx.y * rows;
    const int nrows = min(rows, P.n1b - row0);
    const int per_row = P.nN * L::kN;
    float2 *s_r1 = s_coef + rows * per_row;
    for (int k = threadIdx.x; k < nrows * per_row; k += kDfThreads)
        s_coef[k] = P.poly[(int64_t)row0 * per_row + k];
    for (int k = threadIdx.x; k < nrows * 3; k += kDfThreads) {
        const int r = k / 3, c = k % 3;
        const df::D v = df::from_double(P.r1[3 * (int64_t)(P.i0 + row0 + r) + c]);
        s_r1[k] = make_float2(v.hi, v.lo);
    }
    __syncthreads();

    const int j = blockIdx.x * kDfThreads + threadIdx.x;
    if (j >= P.n2)
        return;
    const float2 x2 = P.r2d[j], y2 = P.r2d[P.n2 + j], z2 = P.r2d[2 * (int64_t)P.n2 + j];
    const df::D a = df::make(P.a_ee_hi, P.a_ee_lo);

    for (int r = 0; r < nrows; r++) {
        const float2 *rr = s_r1 + 3 * r;
        df::D dx = df::sub(df::make(rr[0].x, rr[0].y), df::make(x2.x, x2.y));
        df::D dy = df::sub(df::make(rr[1].x, rr[1].y), df::make(y2.x, y2.y));
        df::D dz = df::sub(df::make(rr[2].x, rr[2].y), df::make(z2.x, z2.y));
        df::D d2 = df::add(df::add(df::sqr(dx), df::sqr(dy)), df::sqr(dz));
        const int64_t o = (int64_t)(row0 + r) * P.ldg + j;
        float2 w4[4];
        bool coalesced = false;
        if (d2.hi < kNearPairR2) {
            // near e-e coalescence the differences are taken in FP64, where they are exact
            // (the coordinates' double-float forms keep only 48 bits); only g12 and its
            // gradient depend on them.  The reference's guard, r12^2 <= 1e-15
            // (src/jast_bh.cu:143), gives g = 0.
            const double *a1 = P.r1 + 3 * (int64_t)(P.i0 + row0 + r);
            const double *a2 = P.r2 + 3 * (int64_t)j;
            const double ex = a1[0] - a2[0], ey = a1[1] - a2[1], ez = a1[2] - a2[2];
            dx = df::from_double(ex);
            dy = df::from_double(ey);
            dz = df::from_double(ez);
            d2 = df::add(df::add(df::sqr(dx), df::sqr(dy)), df::sqr(dz));
            coalesced = !(ex * ex + ey * ey + ez * ez > 1e-15);
        }
        {
            // g = a r / (1 + a r), grad g = a / (r (1 + a r)^2) (r1 - r2)
            df::D g = {0.f, 0.f}, gx = {0.f, 0.f}, gy = {0.f, 0.f}, gz = {0.f, 0.f};
            if (!coalesced) {
                const df::D rd = df::sqrt(d2);
                const df::D ar = df::mul(rd, a);
                const df::D t = df::recip(df::add_f(ar, 1.0f));
                g = df::mul(ar, t);
                const df::D s = df::mul(df::mul(df::sqr(t), a), df::recip(rd));
                gx = df::mul(s, dx);
                gy = df::mul(s, dy);
                gz = df::mul(s, dz);
            }

            df::D ux = {0.f, 0.f}, uy = {0.f, 0.f}, uz = {0.f, 0.f}, dudg = {0.f, 0.f};
            const float2 *cr = s_coef + r * per_row;
            if constexpr (Sp) {
                const df::D g2 = df::sqr(g);
                for (int A = 0; A < P.nN; A++) {
                    const float2 f2v = P.f2d[(int64_t)A * P.n2 + j];
                    const df::D f2 = df::make(f2v.x, f2v.y);
                    const df::D f22 = df::sqr(f2);
                    const float2 *U = cr + A * L::kN;
                    const float2 *W = U + L::kU;
                    auto u = [&](int b, int o) { return df::make(U[b * 5 + o].x, U[b * 5 + o].y); };
                    auto w = [&](int b, int o) { return df::make(W[b * 4 + o].x, W[b * 4 + o].y); };
                    auto pu = [&](int b) {
                        return df::fma(df::fma(df::fma(u(b, 4), g, u(b, 3)), g, u(b, 2)), g2, u(b, 0));
                    };
                    auto pw = [&](int b) { return df::fma(df::fma(w(b, 3), g, w(b, 2)), g, w(b, 1)); };
                    const df::D acc =
                        df::fma(df::fma(df::fma(pu(4), f2, pu(3)), f2, pu(2)), f22, pu(0));
                    const df::D acw =
                        df::fma(df::fma(df::fma(pw(4), f2, pw(3)), f2, pw(2)), f22, pw(0));
                    const float2 *gf = W + L::kW;
                    ux = df::fma(acc, df::make(gf[0].x, gf[0].y), ux);
                    uy = df::fma(acc, df::make(gf[1].x, gf[1].y), uy);
                    uz = df::fma(acc, df::make(gf[2].x, gf[2].y), uz);
                    dudg = df::add(dudg, acw);
                }
                dudg = df::mul(dudg, g);
            } else {
            for (int A = 0; A < P.nN; A++) {
                const float2 f2v = P.f2d[(int64_t)A * P.n2 + j];
                const df::D f2 = df::make(f2v.x, f2v.y);
                const float2 *U = cr + A * L::kN;
                const float2 *W = U + L::kU;
                // du/df1A = sum_b f2^b (sum_o U[b][o] g^o)
                df::D acc = {0.f, 0.f};
    #pragma unroll
                for (int b = E; b >= 0; b--) {
                    df::D in = df::make(U[b * (E + 1) + E].x, U[b * (E + 1) + E].y);
    #pragma unroll
                    for (int q = E - 1; q >= 0; q--)
                        in = df::fma(in, g, df::make(U[b * (E + 1) + q].x, U[b * (E + 1) + q].y));
                    acc = (b == E) ? in : df::fma(acc, f2, in);
                }
                // du/dg contribution = sum_b f2^b (sum_o' W[b][o'] g^o')
                df::D acw = {0.f, 0.f};
    #pragma unroll
                for (int b = E; b >= 0; b--) {
                    df::D in = df::make(W[b * E + E - 1].x, W[b * E + E - 1].y);
    #pragma unroll
                    for (int q = E - 2; q >= 0; q--)
                        in = df::fma(in, g, df::make(W[b * E + q].x, W[b * E + q].y));
                    acw = (b == E) ? in : df::fma(acw, f2, in);
                }
                const float2 *gf = W + L::kW;
                ux = df::fma(acc, df::make(gf[0].x, gf[0].y), ux);
                uy = df::fma(acc, df::make(gf[1].x, gf[1].y), uy);
                uz = df::fma(acc, df::make(gf[2].x, gf[2].y), uz);
                dudg = df::add(dudg, acw);
            }
            }
            ux = df::fma(dudg, gx, ux);
            uy = df::fma(dudg, gy, uy);
            uz = df::fma(dudg, gz, uz);
            const df::D n2v = df::add(df::add(df::sqr(ux), df::sqr(uy)), df::sqr(uz));
            const df::D l = df::mul_f(n2v, -0.5f);
            w4[0] = make_float2(ux.hi, ux.lo);
            w4[1] = make_float2(uy.hi, uy.lo);
            w4[2] = make_float2(uz.hi, uz.lo);
            w4[3] = make_float2(l.hi, l.lo);
        }
#pragma unroll
        for (int c = 0; c < 4; c++)
            P.G[o + c * P.plane] = w4[c];
        if (P.rmax) {
            // row maxima for the slicer, which needs only an exponent e with
            // |G| < 2^e: the high word of the double |hi| (hi + lo rounds to hi,
            // so |hi + lo| never has a larger exponent), built from the float's
            // bits with integer operations -- no FP64 on GB300's slow FP64 pipe.
            // Float subnormals count as 2^-126.  One atomic per converged lane
            // group and row.
            const unsigned mask = __activemask();
            const bool leader = (int)(threadIdx.x & 31) == __ffs(mask) - 1;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const unsigned fb = __float_as_uint(w4[c].x) & 0x7fffffffu;
                const unsigned m = rmax_word(__reduce_max_sync(mask, fb));
                if (leader && m)
                    atomicMax(&P.rmax[(int64_t)c * P.n1b + row0 + r], (unsigned long long)m << 32);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// FP64 operands of the tensor-core pair terms (exponents in {0, 2, 3, 4})
//
// For fixed (r1, r2) the nucleus sum of the sparse-power form is linear in the
// powers f2_A(r2)^b, b in {0, 2, 3, 4}: with k = 4 A + q (b = kPowB[q])
//   V_c(r1, r2) = sum_k C[(r1, c)][k] F[r2][k],   F[r2][k] = f2_A(r2)^b,
//   C[(r1, c)][k] = U_A[b][o](r1) (d f1_A / dx)(r1)   c = 0..3,  o = kPowB[c]
//                   ... d/dy for c = 4..7, d/dz for c = 8..11
//                   W_A[b][o'](r1), o' = c - 11           c = 12..14
//                   0                                     c = 15
// and then, per pair (g = g12 and its gradient, as in pair_df_kernel),
//   grad1 u = sum_o g^o V_{.,o} + g (V_12 + g (V_13 + g V_14)) grad g.
// The contraction over k runs on the tensor cores (split.cu, pair_tc_kernel).
// ---------------------------------------------------------------------------
__constant__ int kPowB[4] = {0, 2, 3, 4};

// F[j * 4 nN + 4 A + q] = f2[A n2 + j]^b_q, FP64
__global__ void pair_tc_f_kernel(int n2, int nN, const double *__restrict__ f2,
                                 double *__restrict__ F)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n2 * nN)
        return;
    const int j = (int)(idx / nN), A = (int)(idx % nN);
    const double f = f2[(int64_t)A * n2 + j];
    const double f2v = f * f;
    double *o = F + (int64_t)j * 4 * nN + 4 * A;
    o[0] = 1.0;
    o[1] = f2v;
    o[2] = f2v * f;
    o[3] = f2v * f2v;
}

// C[((i 16 + c) 4 nN) + 4 A + q] for rows i of the tile, FP64; the polynomial
// coefficients U, W are formed as in r1_poly_kernel<4>.  Also the tile's r1 points in
// double-float, r1d[3 i + c].
__global__ void pair_tc_coef_kernel(int i0, int n, int nN, const double *__restrict__ r1,
                                    const double *__restrict__ rn, double a_en,
                                    const double *__restrict__ tcoef,
                                    const int *__restrict__ texps, const int *__restrict__ toff,
                                    double *__restrict__ C, float2 *__restrict__ r1d)
{
    constexpr int E = 4;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * nN)
        return;
    const int i = (int)(idx / nN), A = (int)(idx % nN);
    const double *p = r1 + 3 * (int64_t)(i0 + i);
    if (A == 0)
        for (int c = 0; c < 3; c++) {  // the point in double-float, for the pair epilogue
            const df::D v = df::from_double(p[c]);
            r1d[3 * (int64_t)i + c] = make_float2(v.hi, v.lo);
        }
    const double dx = p[0] - rn[3 * A], dy = p[1] - rn[3 * A + 1], dz = p[2] - rn[3 * A + 2];
    const double d2 = dx * dx + dy * dy + dz * dz;
    double f = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
    if (d2 > 1e-15) {
        const double d = sqrt(d2);
        const double t = 1.0 / (1.0 + a_en * d);
        f = a_en * d * t;
        const double sg = a_en * t * t / d;
        gx = sg * dx;
        gy = sg * dy;
        gz = sg * dz;
    }
    double F[E + 1];
    F[0] = 1.0;
    for (int k = 1; k <= E; k++)
        F[k] = F[k - 1] * f;
    double U[(E + 1) * (E + 1)], W[(E + 1) * E];
    for (int k = 0; k < (E + 1) * (E + 1); k++)
        U[k] = 0.0;
    for (int k = 0; k < (E + 1) * E; k++)
        W[k] = 0.0;
    for (int k = toff[A]; k < toff[A + 1]; k++) {
        const int e = texps[k];
        const int m = e & 7, nn = (e >> 3) & 7, o = (e >> 6) & 7;
        const double cm = tcoef[3 * k], cn = tcoef[3 * k + 1], co = tcoef[3 * k + 2];
        if (m > 0)
            U[nn * (E + 1) + o] += cm * F[m - 1];
        if (nn > 0)
            U[m * (E + 1) + o] += cn * F[nn - 1];
        if (o > 0) {
            W[nn * E + o - 1] += co * F[m];
            W[m * E + o - 1] += co * F[nn];
        }
    }
    const int64_t K = 4 * (int64_t)nN;
    double *row = C + (int64_t)i * 16 * K + 4 * A;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int b = kPowB[q];
#pragma unroll
        for (int oi = 0; oi < 4; oi++) {
            const double u = U[b * (E + 1) + kPowB[oi]];
            row[oi * K + q] = u * gx;
            row[(4 + oi) * K + q] = u * gy;
            row[(8 + oi) * K + q] = u * gz;
        }
#pragma unroll
        for (int op = 0; op < 3; op++)
            row[(12 + op) * K + q] = W[b * E + op + 1];
        row[15 * K + q] = 0.0;
    }
}

int launch_pair_tc_f(cudaStream_t st, int n2, int nN, const double *f2, double *F)
{
    const int64_t total = (int64_t)n2 * nN;
    if (total == 0)
        return CUTC_OK;
    pair_tc_f_kernel<<<ceil_div(total, 256), 256, 0, st>>>(n2, nN, f2, F);
    CUTC_CUDA_TRY(cudaGetLastError());
    return CUTC_OK;
}

int launch_pair_tc_coef(cudaStream_t st, int i0, int n, int nN, const double *r1, const double *rn,
                        double a_en, const double *coef, const int *exps, const int *term_off,
                        double *C, float2 *r1d)
{
    const int64_t total = (int64_t)n * nN;
    if (total == 0)
        return CUTC_OK;
    pair_tc_coef_kernel<<<ceil_div(total, 128), 128, 0, st>>>(i0, n, nN, r1, rn, a_en, coef,
                                                              exps, term_off, C, r1d);
    CUTC_CUDA_TRY(cudaGetLastError());
    return CUTC_OK;
}

__global__ void f64_to_df_kernel(double *x, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const df::D v = df::from_double(x[i]);
        reinterpret_cast<float2 *>(x)[i] = make_float2(v.hi, v.lo);
    }
}

int launch_f64_to_df(cudaStream_t st, double *x, int64_t n)
{
    f64_to_df_kernel<<<4 * 152, 256, 0, st>>>(x, n);
    CUTC_CUDA_TRY(cudaGetLastError());
    return CUTC_OK;
}

int pair_df_max_exp(const int *exps, int n_terms)
{
    int E = 0;
    for (int k = 0; k < n_terms; k++) {
        const int e = exps[k];
        E = max(E, max(e & 7, max((e >> 3) & 7, (e >> 6) & 7)));
    }
    return E <= 4 ? 4 : 6;
}

bool pair_df_sparse(const int *exps, int n_terms)
{
    for (int k = 0; k < n_terms; k++) {
        const int e = exps[k];
        const int m = e & 7, n = (e >> 3) & 7, o = (e >> 6) & 7;
        if (m == 1 || n == 1 || o == 1 || m > 4 || n > 4 || o > 4)
            return false;
    }
    return true;
}

size_t pair_df_poly_bytes(int E, int n1b, int nN)
{
    const int kN = E == 4 ? PolyLayout<4>::kN : PolyLayout<6>::kN;
    return (size_t)n1b * nN * kN * sizeof(float2);
}

int launch_r2_df(cudaStream_t st, int n2, int nN, const double *r2, const double *f2, float2 *r2d,
                 float2 *f2d)
{
    r2_df_kernel<<<ceil_div(n2, 256), 256, 0, st>>>(n2, nN, r2, f2, r2d, f2d);
    CUTC_CUDA_TRY(cudaGetLastError());
    return CUTC_OK;
}

template <int E, bool Sp>
static int launch_df_impl(cudaStream_t st, PairDfArgs P, const double *rn, double a_en)
{
    using L = PolyLayout<E>;
    const int64_t total = (int64_t)P.n1b * P.nN;
    r1_poly_kernel<E><<<ceil_div(total, 128), 128, 0, st>>>(P.i0, P.n1b, P.nN, P.r1, rn, a_en,
                                                            P.coef, P.exps, P.term_off, P.poly_w);
    CUTC_CUDA_TRY(cudaGetLastError());
    const size_t per_row = (size_t)P.nN * L::kN * sizeof(float2) + 3 * sizeof(float2);
    const size_t budget = 160 * 1024;
    int rows = (int)std::min<size_t>(8, budget / per_row);
    if (rows < 1) {
        cutc_set_error(CUTC_ERR_INVALID, "too many nuclei for the df pair kernel");
        return CUTC_ERR_INVALID;
    }
    P.rows_per_cta = rows;
    const size_t smem = rows * per_row;
    static std::atomic<unsigned long long> attr_done{0};
    const unsigned long long bit = current_device_bit();
    if (!(attr_done.load() & bit)) {
        CUTC_CUDA_TRY(cudaFuncSetAttribute(pair_df_kernel<E, Sp>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        attr_done.fetch_or(bit);
    }
    dim3 grid(ceil_div(P.n2, kDfThreads), ceil_div(P.n1b, rows));
    pair_df_kernel<E, Sp><<<grid, kDfThreads, smem, st>>>(P);
    CUTC_CUDA_TRY(cudaGetLastError());
    return CUTC_OK;
}

int launch_pair_df(cudaStream_t st, const PairDfArgs &P, int E, bool sparse, const double *rn,
                   double a_en)
{
    if (P.n1b <= 0 || P.n2 <= 0)
        return CUTC_OK;
    if (E == 4)
        return sparse ? launch_df_impl<4, true>(st, P, rn, a_en)
                      : launch_df_impl<4, false>(st, P, rn, a_en);
    return launch_df_impl<6, false>(st, P, rn, a_en);
}

}  // namespace cutc
