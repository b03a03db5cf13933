/*
 * CPU oracle for the cutc_int hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is the checker that the GPU engine is compared against, and the
 * CPU baseline timed by bench.py.  It is never linked into, called by or
 * shipped with the product library.
 *
 * It restates, in plain FP64 C with OpenMP, the arithmetic of the reference
 * CuTC kernels (the reference has no CPU path):
 *
 *   oracle_pair            src/jast_bh.cu:115-254  (cutc_int_bh_kernel, powd_int :3-28)
 *   oracle_long_range      src/long_range_integ.cu:21-45 (int_long_range_kernel)
 *   oracle_short_herm      src/short_range_integ_herm.cu:20-44
 *   oracle_short_nonherm   src/short_range_integ_nonherm.cu:23-63
 *   oracle_add_trans       src/add_trans_inplace.cu:12-13 (A <- A + A^T)
 *
 * The dense contractions (cuBLAS DGEMM in the reference,
 * src/build_int2_grad1_u12_ao.cu:152-159 and src/build_int_2e_ao.cu:60-67,97-104)
 * are done by the Python driver oracle/oracle.py with numpy matmul.
 *
 * The a_en / a_ee scale factors generalise the reference's fixed
 * r/(1+r) (src/jast_bh.cu:145,171,191) to a r/(1 + a r); a = 1 reproduces it.
 *
 * Layouts are the reference's Fortran column-major ones
 * (src/cutc_module.f90:24-35): r(3,n), aos(n,nA,4), c/m/n/o_bh(nB,nN).
 * Compiled with -ffp-contract=off so results do not depend on whether the
 * host compiler fuses multiply-adds.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>

/* a^b for b in [0,6] by repeated multiplication (src/jast_bh.cu:3-28). */
static inline double pow_small(double a, int b)
{
    double a2;
    switch (b) {
    case 0: return 1.0;
    case 1: return a;
    case 2: return a * a;
    case 3: return a * a * a;
    case 4: a2 = a * a; return a2 * a2;
    case 5: a2 = a * a; return a * a2 * a2;
    case 6: a2 = a * a; return a2 * a2 * a2;
    default: return NAN; /* the reference leaves this undefined */
    }
}

/* f(r) = a r / (1 + a r) and its radial factor f'(r)/r, with the reference's
 * coalescence guard r^2 > 1e-15 (src/jast_bh.cu:143,169). */
static inline void scaled_dist(double dx, double dy, double dz, double a,
                               double *f, double *gx, double *gy, double *gz)
{
    double d2 = dx * dx + dy * dy + dz * dz;
    if (d2 > 1e-15) {
        double d = sqrt(d2);
        double t = 1.0 / (1.0 + a * d);
        *f = a * d * t;
        double s = a * t * t / d;
        *gx = s * dx;
        *gy = s * dy;
        *gz = s * dz;
    } else {
        *f = 0.0;
        *gx = *gy = *gz = 0.0;
    }
}

/*
 * grad1 u(r1, r2) for r1 in [i0, i0 + n1b) and every r2:
 *   G[c][i][j], c = 0..2 the gradient components, c = 3 the value
 *   -1/2 |grad1 u|^2; i in [0, n1b), j in [0, n2); j fastest
 *   (layout of grad1_u12 in src/jast_bh.cu:113,129-131,252).
 * Terms with |c| < 1e-10 are skipped (src/jast_bh.cu:203).
 */
void oracle_pair(int i0, int n1b, int n2, int n_nuc, int size_bh,
                 const double *r1, const double *r2, const double *rn,
                 const double *c_bh, const int *m_bh, const int *n_bh, const int *o_bh,
                 double a_en, double a_ee, double *G)
{
    const size_t plane = (size_t)n1b * (size_t)n2;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < n1b; i++) {
        const double x1 = r1[3 * (size_t)(i0 + i) + 0];
        const double y1 = r1[3 * (size_t)(i0 + i) + 1];
        const double z1 = r1[3 * (size_t)(i0 + i) + 2];
        for (int j = 0; j < n2; j++) {
            const double x2 = r2[3 * (size_t)j + 0];
            const double y2 = r2[3 * (size_t)j + 1];
            const double z2 = r2[3 * (size_t)j + 2];
            double g, gx, gy, gz;
            scaled_dist(x1 - x2, y1 - y2, z1 - z2, a_ee, &g, &gx, &gy, &gz);
            double ux = 0.0, uy = 0.0, uz = 0.0;
            for (int A = 0; A < n_nuc; A++) {
                const double xa = rn[3 * A + 0], ya = rn[3 * A + 1], za = rn[3 * A + 2];
                double f1, f1x, f1y, f1z, f2 = 0.0;
                scaled_dist(x1 - xa, y1 - ya, z1 - za, a_en, &f1, &f1x, &f1y, &f1z);
                {
                    /* e2-n term: a r / (1 + a r) as one division (src/jast_bh.cu:185-194) */
                    const double dx = x2 - xa, dy = y2 - ya, dz = z2 - za;
                    const double d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 > 1e-15) {
                        const double d = a_en * sqrt(d2);
                        f2 = d / (1.0 + d);
                    }
                }
                for (int p = 0; p < size_bh; p++) {
                    const int k = p + size_bh * A;
                    const double c = c_bh[k];
                    if (fabs(c) < 1e-10)
                        continue;
                    const int m = m_bh[k], n = n_bh[k], o = o_bh[k];
                    /* src/jast_bh.cu:209-242 */
                    double f1_m = 1.0, f2_m = 1.0, f1_mm1 = 0.0;
                    if (m > 0) {
                        f1_mm1 = pow_small(f1, m - 1);
                        f1_m = f1_mm1 * f1;
                        f2_m = pow_small(f2, m);
                    }
                    double f1_n = 1.0, f2_n = 1.0, f1_nm1 = 0.0;
                    if (n > 0) {
                        f1_nm1 = pow_small(f1, n - 1);
                        f1_n = f1_nm1 * f1;
                        f2_n = pow_small(f2, n);
                    }
                    double t1 = 0.0, t2 = 0.0;
                    if (m > 0)
                        t1 += (double)m * f1_mm1 * f2_n;
                    if (n > 0)
                        t1 += (double)n * f1_nm1 * f2_m;
                    if (o > 0) {
                        const double g_om1 = pow_small(g, o - 1);
                        const double g_o = g_om1 * g;
                        t2 = c * (double)o * g_om1 * (f1_m * f2_n + f1_n * f2_m);
                        t1 = c * t1 * g_o;
                    } else {
                        t1 *= c;
                    }
                    ux += t1 * f1x + t2 * gx;
                    uy += t1 * f1y + t2 * gy;
                    uz += t1 * f1z + t2 * gz;
                }
            }
            const size_t q = (size_t)i * n2 + j;
            G[q] = ux;
            G[q + plane] = uy;
            G[q + 2 * plane] = uz;
            G[q + 3 * plane] = -0.5 * (ux * ux + uy * uy + uz * uz);
        }
    }
}

/*
 * P[(j + nA i) * n2 + g] = w2[g] chi_i(g) chi_j(g) for g in [g0, g0 + n2b)
 * (src/long_range_integ.cu:39; column-major (n2b, nA^2), column j + nA i).
 * aos2 is the full (n2, nA, 4) array; only the value component is read.
 */
void oracle_long_range(int g0, int n2b, int n2, int n_ao, const double *w2,
                       const double *aos2, double *P)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n_ao; i++) {
        for (int j = 0; j < n_ao; j++) {
            double *col = P + (size_t)(j + n_ao * i) * n2b;
            const double *ci = aos2 + (size_t)n2 * i + g0;
            const double *cj = aos2 + (size_t)n2 * j + g0;
            for (int g = 0; g < n2b; g++)
                col[g] = w2[g0 + g] * ci[g] * cj[g];
        }
    }
}

/* S0[(j + nA i) * n1 + g] = w1 chi_i chi_j (src/short_range_integ_herm.cu:38). */
void oracle_short_herm(int n1, int n_ao, const double *w1, const double *aos1, double *S0)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n_ao; i++) {
        for (int j = 0; j < n_ao; j++) {
            double *col = S0 + (size_t)(j + n_ao * i) * n1;
            const double *ci = aos1 + (size_t)n1 * i;
            const double *cj = aos1 + (size_t)n1 * j;
            for (int g = 0; g < n1; g++)
                col[g] = w1[g] * ci[g] * cj[g];
        }
    }
}

/*
 * S[(j + nA i) * 3 n1 + m n1 + g] = w1 (chi_j d_m chi_i - chi_i d_m chi_j)
 * (src/short_range_integ_nonherm.cu:55; column-major (3 n1, nA^2)).
 */
void oracle_short_nonherm(int n1, int n_ao, const double *w1, const double *aos1, double *S)
{
    const size_t na1 = (size_t)n_ao * n1;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n_ao; i++) {
        for (int j = 0; j < n_ao; j++) {
            double *col = S + (size_t)(j + n_ao * i) * 3 * n1;
            const double *vi = aos1 + (size_t)n1 * i;
            const double *vj = aos1 + (size_t)n1 * j;
            for (int m = 0; m < 3; m++) {
                const double *di = vi + (m + 1) * na1;
                const double *dj = vj + (m + 1) * na1;
                for (int g = 0; g < n1; g++)
                    col[(size_t)m * n1 + g] = w1[g] * (vj[g] * di[g] - vi[g] * dj[g]);
            }
        }
    }
}

/* A <- A + A^T for a square n x n matrix (src/add_trans_inplace.cu:12-13). */
void oracle_add_trans(int64_t n, double *A)
{
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; i++) {
        for (int64_t j = 0; j <= i; j++) {
            double s = A[i + n * j] + A[j + n * i];
            A[i + n * j] = s;
            A[j + n * i] = s;
        }
    }
}
