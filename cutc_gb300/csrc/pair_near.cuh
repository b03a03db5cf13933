// The pair terms of one (r1, r2) pair in FP64, for pairs near e-e coalescence
// (shared by the double-float and the tensor-core pair kernels).
#pragma once

#include "common.cuh"
#include "pair.cuh"

namespace cutc {

// r12^2 below which a pair of the split form's pair kernels is evaluated in FP64
constexpr float kNearPairR2 = 1.0e-4f;

// One pair in FP64, term by term as the reference kernel does it
// (src/jast_bh.cu:138-254), for pairs near e-e coalescence.
static __device__ __noinline__ void pair_fp64_single(const PairDfArgs &P, int i, int j, double out[4])
{
    const int64_t gi = P.i0 + i;
    const double dx = P.r1[3 * gi] - P.r2[3 * (int64_t)j];
    const double dy = P.r1[3 * gi + 1] - P.r2[3 * (int64_t)j + 1];
    const double dz = P.r1[3 * gi + 2] - P.r2[3 * (int64_t)j + 2];
    const double d2 = dx * dx + dy * dy + dz * dz;
    const double a = P.a_ee;
    double g = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
    if (d2 > 1e-15) {
        const double d = sqrt(d2);
        const double t = 1.0 / (1.0 + a * d);
        g = a * d * t;
        const double s = a * t * t / d;
        gx = s * dx;
        gy = s * dy;
        gz = s * dz;
    }
    double ux = 0.0, uy = 0.0, uz = 0.0;
    for (int A = 0; A < P.nN; A++) {
        const NucTerm t1 = P.t1[(int64_t)i * P.nN + A];
        const double f1 = t1.f, f2 = P.f2[(int64_t)A * P.n2 + j];
        for (int k = P.term_off[A]; k < P.term_off[A + 1]; k++) {
            const int e = P.exps[k];
            const int m = e & 7, n = (e >> 3) & 7, o = (e >> 6) & 7;
            double F1[kMaxExp + 1], F2[kMaxExp + 1], Gp[kMaxExp + 1];
            F1[0] = F2[0] = Gp[0] = 1.0;
            for (int q = 1; q <= kMaxExp; q++) {
                F1[q] = F1[q - 1] * f1;
                F2[q] = F2[q - 1] * f2;
                Gp[q] = Gp[q - 1] * g;
            }
            double t1v = 0.0, t2v = 0.0;
            if (m > 0)
                t1v += P.coef[3 * k] * F1[m - 1] * F2[n];
            if (n > 0)
                t1v += P.coef[3 * k + 1] * F1[n - 1] * F2[m];
            t1v *= Gp[o];
            if (o > 0)
                t2v = P.coef[3 * k + 2] * Gp[o - 1] * (F1[m] * F2[n] + F1[n] * F2[m]);
            ux += t1v * t1.gx + t2v * gx;
            uy += t1v * t1.gy + t2v * gy;
            uz += t1v * t1.gz + t2v * gz;
        }
    }
    out[0] = ux;
    out[1] = uy;
    out[2] = uz;
    out[3] = -0.5 * (ux * ux + uy * uy + uz * uz);
}

}  // namespace cutc
