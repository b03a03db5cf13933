// Atomic orbitals on the grids, evaluated on the device from a basis.
//
// The reference takes AO values and gradients on both grids from its caller
// (src/cutc_module.f90:28-29: aos_data1(n_grid1, n_ao, 4), aos_data2(n_grid2,
// n_ao, 4)); a request can instead name the basis and have them computed here.
// A basis is a list of Cartesian contracted Gaussians, one entry per AO:
//     chi_a(r) = x^lx y^ly z^lz sum_k c_k exp(-alpha_k |r - C_a|^2),
// (x, y, z) = r - C_a, normalisation folded into the c_k.  Values and the three
// gradient components are written in the reference layout, one thread per
// (point, AO), consecutive threads on consecutive points.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "aos.cuh"
#include "common.cuh"

namespace cutc {

__device__ __forceinline__ double ipow(double x, int k)
{
    double v = 1.0;
    for (int i = 0; i < k; i++)
        v *= x;
    return v;
}

// out[(c * nA + a) * ld + g] for c < comps (value, d/dx, d/dy, d/dz)
__global__ void eval_aos_kernel(int n, const double *__restrict__ r, BasisDev B, int comps,
                                double *__restrict__ out, int64_t ld)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int a = blockIdx.y;
    if (g >= n)
        return;
    const double x = r[3 * (int64_t)g] - B.center[3 * a];
    const double y = r[3 * (int64_t)g + 1] - B.center[3 * a + 1];
    const double z = r[3 * (int64_t)g + 2] - B.center[3 * a + 2];
    const double r2 = x * x + y * y + z * z;
    double rad = 0.0, drad = 0.0;  // radial part and its derivative in r^2
    for (int k = B.offset[a]; k < B.offset[a + 1]; k++) {
        const double e = B.coef[k] * exp(-B.exp[k] * r2);
        rad += e;
        drad -= B.exp[k] * e;
    }
    const int lx = B.power[3 * a], ly = B.power[3 * a + 1], lz = B.power[3 * a + 2];
    const double px = ipow(x, lx), py = ipow(y, ly), pz = ipow(z, lz);
    const double ang = px * py * pz;
    const int64_t plane = (int64_t)B.n_ao * ld;
    out[(int64_t)a * ld + g] = ang * rad;
    if (comps == 4) {
        const double dpx = lx ? lx * ipow(x, lx - 1) : 0.0;
        const double dpy = ly ? ly * ipow(y, ly - 1) : 0.0;
        const double dpz = lz ? lz * ipow(z, lz - 1) : 0.0;
        out[plane + (int64_t)a * ld + g] = dpx * py * pz * rad + ang * 2.0 * x * drad;
        out[2 * plane + (int64_t)a * ld + g] = px * dpy * pz * rad + ang * 2.0 * y * drad;
        out[3 * plane + (int64_t)a * ld + g] = px * py * dpz * rad + ang * 2.0 * z * drad;
    }
}

int validate_basis(const cutc_basis *b, int n_ao)
{
    if (!b || b->n_ao != n_ao || n_ao <= 0 || !b->center || !b->power || !b->prim_offset ||
        !b->prim_exp || !b->prim_coef) {
        cutc_set_error(CUTC_ERR_INVALID, "basis missing or not of %d functions", n_ao);
        return CUTC_ERR_INVALID;
    }
    if (n_ao > 65535) {
        cutc_set_error(CUTC_ERR_INVALID, "basis of %d functions exceeds 65535", n_ao);
        return CUTC_ERR_INVALID;
    }
    if (b->prim_offset[0] != 0) {
        cutc_set_error(CUTC_ERR_INVALID, "basis prim_offset[0] must be 0");
        return CUTC_ERR_INVALID;
    }
    for (int a = 0; a < n_ao; a++) {
        const int np = b->prim_offset[a + 1] - b->prim_offset[a];
        if (np < 1 || np > kMaxPrim) {
            cutc_set_error(CUTC_ERR_INVALID, "AO %d has %d primitives (1..%d allowed)", a, np,
                           kMaxPrim);
            return CUTC_ERR_INVALID;
        }
        for (int c = 0; c < 3; c++)
            if (b->power[3 * a + c] < 0 || b->power[3 * a + c] > kMaxAoPower) {
                cutc_set_error(CUTC_ERR_INVALID, "AO %d has a Cartesian power outside [0, %d]", a,
                               kMaxAoPower);
                return CUTC_ERR_INVALID;
            }
    }
    return CUTC_OK;
}

int upload_basis(Workspace &W, int slot, cudaStream_t st, const cutc_basis *b, BasisDev *out)
{
    const int nA = b->n_ao, np = b->prim_offset[nA];
    // doubles first (centres, exponents, coefficients), then ints (powers, offsets)
    const size_t nd = 3 * (size_t)nA + 2 * (size_t)np, ni = 3 * (size_t)nA + nA + 1;
    std::vector<unsigned char> h(nd * 8 + ni * 4);
    double *hd = reinterpret_cast<double *>(h.data());
    int *hi = reinterpret_cast<int *>(h.data() + nd * 8);
    std::copy(b->center, b->center + 3 * (size_t)nA, hd);
    std::copy(b->prim_exp, b->prim_exp + np, hd + 3 * (size_t)nA);
    std::copy(b->prim_coef, b->prim_coef + np, hd + 3 * (size_t)nA + np);
    std::copy(b->power, b->power + 3 * (size_t)nA, hi);
    std::copy(b->prim_offset, b->prim_offset + nA + 1, hi + 3 * (size_t)nA);
    void *p;
    CUTC_TRY(W.get(slot, h.size(), &p));
    CUTC_CUDA_TRY(cudaMemcpyAsync(p, h.data(), h.size(), cudaMemcpyHostToDevice, st));
    CUTC_CUDA_TRY(cudaStreamSynchronize(st));  // h goes out of scope
    const double *dd = (const double *)p;
    const int *di = (const int *)((const unsigned char *)p + nd * 8);
    out->n_ao = nA;
    out->center = dd;
    out->exp = dd + 3 * (size_t)nA;
    out->coef = dd + 3 * (size_t)nA + np;
    out->power = di;
    out->offset = di + 3 * (size_t)nA;
    return CUTC_OK;
}

int launch_eval_aos(cudaStream_t st, const BasisDev &B, int n, const double *r, int comps,
                    double *out, int64_t ld)
{
    if (n <= 0)
        return CUTC_OK;
    dim3 grid(ceil_div(n, 128), (unsigned)B.n_ao);
    eval_aos_kernel<<<grid, 128, 0, st>>>(n, r, B, comps, out, ld);
    CUTC_CUDA_TRY(cudaGetLastError());
    note_launches(1);
    return CUTC_OK;
}

}  // namespace cutc
