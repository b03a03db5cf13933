// Boys-Handy Jastrow pair terms grad1 u(r1, r2) on sm_103a (plain FP64 form).
//
// Computes, for every (r1, r2) pair of a tile, the quantity of the reference
// kernel cutc_int_bh_kernel (src/jast_bh.cu:31-264):
//
//   u(r1, r2) = sum_A sum_p c_pA [f1A^m f2A^n + f1A^n f2A^m] g12^o
//   f = a_en r / (1 + a_en r),  g12 = a_ee r12 / (1 + a_ee r12)
//   G[0..2] = grad1 u,  G[3] = -1/2 |grad1 u|^2
//
// Restructured for the GPU instead of transcribed:
//   * f1A, grad f1A (per r1 point) and f2A (per r2 point) are computed once
//     per point by small kernels, not once per pair and term;
//   * per pair and nucleus the terms reduce to two scalars,
//       du/df1A = sum_p c_p g^o (m f1^{m-1} f2^n + n f1^{n-1} f2^m)
//       du/dg  += sum_p c_p o g^{o-1} (f1^m f2^n + f1^n f2^m)
//     and grad1 u = sum_A du/df1A grad f1A + du/dg grad g12, which needs
//     three vector FMAs per nucleus instead of three per term;
//   * powers 0..6 of f1, f2 and g are tabulated in shared memory, so each
//     term costs a handful of table reads and ~9 FP64 operations;
//   * one thread owns one r2 point and walks the CTA's r1 rows, so the G
//     stores of a warp are 32 consecutive doubles (coalesced), unlike the
//     reference's stride-n2 stores.
// Terms with |c| < 1e-10 are dropped on the host (src/jast_bh.cu:203) and the
// coalescence guard r^2 > 1e-15 (src/jast_bh.cu:143,169,189) is kept.
#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "pair.cuh"

namespace cutc {

// ---------------------------------------------------------------------------
// per-point nucleus terms
// ---------------------------------------------------------------------------

// t1[(i * nN + A)] = (f1A, d f1A/dx, d f1A/dy, d f1A/dz) for r1 rows [i0, i0+n)
__global__ void r1_nuclear_terms_kernel(int i0, int n, int nN, const double *__restrict__ r1,
                                        const double *__restrict__ rn, double a,
                                        NucTerm *__restrict__ t1)
{
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * nN)
        return;
    int i = (int)(idx / nN), A = (int)(idx % nN);
    const double *p = r1 + 3 * (int64_t)(i0 + i);
    double dx = p[0] - rn[3 * A], dy = p[1] - rn[3 * A + 1], dz = p[2] - rn[3 * A + 2];
    double d2 = dx * dx + dy * dy + dz * dz;
    NucTerm v = {0.0, 0.0, 0.0, 0.0};
    if (d2 > 1e-15) {
        double d = sqrt(d2);
        double t = 1.0 / (1.0 + a * d);
        double s = a * t * t / d;
        v = {a * d * t, s * dx, s * dy, s * dz};
    }
    t1[idx] = v;
}

// f2[A * n2 + j] = a r / (1 + a r), r = |r2_j - R_A|
__global__ void r2_nuclear_terms_kernel(int n2, int nN, const double *__restrict__ r2,
                                        const double *__restrict__ rn, double a,
                                        double *__restrict__ f2)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    int A = blockIdx.y;
    if (j >= n2)
        return;
    double dx = r2[3 * (int64_t)j] - rn[3 * A];
    double dy = r2[3 * (int64_t)j + 1] - rn[3 * A + 1];
    double dz = r2[3 * (int64_t)j + 2] - rn[3 * A + 2];
    double d2 = dx * dx + dy * dy + dz * dz;
    double f = 0.0;
    if (d2 > 1e-15) {
        double d = a * sqrt(d2);
        f = d / (1.0 + d);
    }
    f2[(int64_t)A * n2 + j] = f;
}

// ---------------------------------------------------------------------------
// the pair kernel
// ---------------------------------------------------------------------------

constexpr int kPairThreads = 256;
constexpr int kPairRows = 8;  // r1 rows per CTA
constexpr int kTab = kMaxExp + 1;

__device__ __forceinline__ void powers(double x, double *t, int stride)
{
    double x2 = x * x;
    t[0] = 1.0;
    t[stride] = x;
    t[2 * stride] = x2;
    t[3 * stride] = x2 * x;
    t[4 * stride] = x2 * x2;
    t[5 * stride] = x2 * x2 * x;
    t[6 * stride] = x2 * x2 * x2;
}

__global__ void __launch_bounds__(kPairThreads)
pair_f64_kernel(PairArgs P)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // shared layout: term coefs (3 doubles/term) | F1 tables | f1 gradients |
    //                per-thread F2 and g tables | term exps | term offsets
    double *s_coef = reinterpret_cast<double *>(smem_raw);
    double *s_f1 = s_coef + 3 * P.n_terms;                  // [row][A][kTab]
    double *s_f1g = s_f1 + kPairRows * P.nN * kTab;         // [row][A][3]
    double *s_f2 = s_f1g + kPairRows * P.nN * 3;            // [kTab][threads]
    double *s_g = s_f2 + kTab * kPairThreads;               // [kTab][threads]
    int *s_exp = reinterpret_cast<int *>(s_g + kTab * kPairThreads);
    int *s_off = s_exp + P.n_terms;

    const int tid = threadIdx.x;
    for (int k = tid; k < P.n_terms; k += kPairThreads) {
        s_coef[3 * k] = P.coef[3 * k];
        s_coef[3 * k + 1] = P.coef[3 * k + 1];
        s_coef[3 * k + 2] = P.coef[3 * k + 2];
        s_exp[k] = P.exps[k];
    }
    for (int k = tid; k <= P.nN; k += kPairThreads)
        s_off[k] = P.term_off[k];
    const int row0 = blockIdx.y * kPairRows;
    const int nrows = min(kPairRows, P.n1b - row0);
    for (int k = tid; k < nrows * P.nN; k += kPairThreads) {
        int r = k / P.nN, A = k % P.nN;
        NucTerm v = P.t1[(int64_t)(row0 + r) * P.nN + A];
        powers(v.f, s_f1 + (r * P.nN + A) * kTab, 1);
        s_f1g[(r * P.nN + A) * 3 + 0] = v.gx;
        s_f1g[(r * P.nN + A) * 3 + 1] = v.gy;
        s_f1g[(r * P.nN + A) * 3 + 2] = v.gz;
    }
    __syncthreads();

    const int j = blockIdx.x * kPairThreads + tid;
    if (j >= P.n2)
        return;
    const double x2 = P.r2[3 * (int64_t)j], y2 = P.r2[3 * (int64_t)j + 1], z2 = P.r2[3 * (int64_t)j + 2];
    double *myF2 = s_f2 + tid;
    double *myG = s_g + tid;
    const double a = P.a_ee;

    for (int r = 0; r < nrows; r++) {
        const int64_t gi = P.i0 + row0 + r;
        const double dx = P.r1[3 * gi] - x2, dy = P.r1[3 * gi + 1] - y2, dz = P.r1[3 * gi + 2] - z2;
        const double d2 = dx * dx + dy * dy + dz * dz;
        double g = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
        if (d2 > 1e-15) {
            double d = sqrt(d2);
            double t = 1.0 / (1.0 + a * d);
            g = a * d * t;
            double s = a * t * t / d;
            gx = s * dx;
            gy = s * dy;
            gz = s * dz;
        }
        powers(g, myG, kPairThreads);
        double ux = 0.0, uy = 0.0, uz = 0.0, dudg = 0.0;
        for (int A = 0; A < P.nN; A++) {
            powers(P.f2[(int64_t)A * P.n2 + j], myF2, kPairThreads);
            const double *F1 = s_f1 + (r * P.nN + A) * kTab;
            double dudf1 = 0.0;
            const int kend = s_off[A + 1];
            for (int k = s_off[A]; k < kend; k++) {
                const int e = s_exp[k];
                const int m = e & 7, n = (e >> 3) & 7, o = (e >> 6) & 7;
                const int mm1 = m > 0 ? m - 1 : 0, nm1 = n > 0 ? n - 1 : 0, om1 = o > 0 ? o - 1 : 0;
                const double cm = s_coef[3 * k], cn = s_coef[3 * k + 1], co = s_coef[3 * k + 2];
                const double F2m = myF2[m * kPairThreads], F2n = myF2[n * kPairThreads];
                // c m f1^{m-1} f2^n + c n f1^{n-1} f2^m   (cm = 0 when m = 0, cn = 0 when n = 0)
                double t1 = cm * F1[mm1] * F2n + cn * F1[nm1] * F2m;
                dudf1 += t1 * myG[o * kPairThreads];
                // c o g^{o-1} (f1^m f2^n + f1^n f2^m)   (co = 0 when o = 0)
                double b = F1[m] * F2n + F1[n] * F2m;
                dudg += co * myG[om1 * kPairThreads] * b;
            }
            const double *fg = s_f1g + (r * P.nN + A) * 3;
            ux += dudf1 * fg[0];
            uy += dudf1 * fg[1];
            uz += dudf1 * fg[2];
        }
        ux += dudg * gx;
        uy += dudg * gy;
        uz += dudg * gz;
        double *out = P.G + (int64_t)(row0 + r) * P.ldg + j;
        out[0] = ux;
        out[P.plane] = uy;
        out[2 * P.plane] = uz;
        out[3 * P.plane] = -0.5 * (ux * ux + uy * uy + uz * uz);
    }
}

size_t pair_f64_smem(int n_terms, int nN)
{
    return sizeof(double) * (3 * (size_t)n_terms + (size_t)kPairRows * nN * (kTab + 3) +
                             2 * (size_t)kTab * kPairThreads) +
           sizeof(int) * ((size_t)n_terms + nN + 1);
}

int launch_r1_terms(cudaStream_t st, int i0, int n, int nN, const double *r1, const double *rn,
                    double a, NucTerm *t1)
{
    int64_t total = (int64_t)n * nN;
    if (total == 0)
        return CUTC_OK;
    r1_nuclear_terms_kernel<<<ceil_div(total, 256), 256, 0, st>>>(i0, n, nN, r1, rn, a, t1);
    CUTC_CUDA_TRY(cudaGetLastError());
    return CUTC_OK;
}

int launch_r2_terms(cudaStream_t st, int n2, int nN, const double *r2, const double *rn,
                    double a, double *f2)
{
    dim3 grid(ceil_div(n2, 256), nN);
    r2_nuclear_terms_kernel<<<grid, 256, 0, st>>>(n2, nN, r2, rn, a, f2);
    CUTC_CUDA_TRY(cudaGetLastError());
    return CUTC_OK;
}

int launch_pair_f64(cudaStream_t st, const PairArgs &P)
{
    if (P.n1b <= 0 || P.n2 <= 0)
        return CUTC_OK;
    size_t smem = pair_f64_smem(P.n_terms, P.nN);
    static std::atomic<unsigned long long> attr_done{0};
    const unsigned long long bit = current_device_bit();
    if (!(attr_done.load() & bit)) {
        CUTC_CUDA_TRY(cudaFuncSetAttribute(pair_f64_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
        attr_done.fetch_or(bit);
    }
    if (smem > 220 * 1024) {
        cutc_set_error(CUTC_ERR_INVALID, "too many nuclei/terms for the pair kernel (%zu B smem)", smem);
        return CUTC_ERR_INVALID;
    }
    dim3 grid(ceil_div(P.n2, kPairThreads), ceil_div(P.n1b, kPairRows));
    pair_f64_kernel<<<grid, kPairThreads, smem, st>>>(P);
    CUTC_CUDA_TRY(cudaGetLastError());
    return CUTC_OK;
}

}  // namespace cutc

// ---------------------------------------------------------------------------
// Allocation-free pair terms
//
// Some callers cannot let a library allocate device memory: host programs
// whose own memory manager has reserved the whole device, and latency-critical
// serving loops in which cudaMalloc / cudaFree would stall on device-wide
// synchronisation.  cutc_jast_bh_dev_noalloc serves them: its scratch (the
// per-point nucleus terms, the r2 e-n terms and the compact Jastrow term
// table) lives in the static array below, sized once at load time, so a call
// allocates nothing -- no cudaMalloc, no cudaFree, no library allocator, no
// engine context.  The caller still provides the inputs and the output.  Each
// call synchronises its stream and reads the status word back.
// ---------------------------------------------------------------------------

namespace cutc {

// Fixed capacity of the scratch: every GPU that loads the library holds it until exit.
constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// layout of the scratch
constexpr size_t kNaStatus = 0;                                       // int status word
constexpr size_t kNaCoef = 256;                                       // double[3 * kMaxTerms]
constexpr size_t kNaExps = kNaCoef + 3 * sizeof(double) * kMaxTerms;  // int[kMaxTerms]
constexpr size_t kNaOff = kNaExps + sizeof(int) * kMaxTerms;          // int[kMaxNuc + 1]
constexpr size_t kNaT1 = (kNaOff + sizeof(int) * (kMaxNuc + 1) + 255) & ~(size_t)255;

// The compact term table built on the device (the same table build_terms makes
// on the host for the allocating entry points): terms with |c| < 1e-10 are
// dropped (src/jast_bh.cu:203); an exponent outside [0, 6] sets the status.
__global__ void noalloc_terms_kernel(int nN, int nB, const double *__restrict__ c,
                                     const int *__restrict__ m, const int *__restrict__ n,
                                     const int *__restrict__ o, double *coef, int *exps, int *off,
                                     int *status)
{
    if (blockIdx.x != 0 || threadIdx.x != 0)
        return;
    int nt = 0;
    for (int A = 0; A < nN; A++) {
        off[A] = nt;
        for (int p = 0; p < nB; p++) {
            const int k = p + nB * A;
            const int mm = m[k], nn = n[k], oo = o[k];
            if (mm < 0 || mm > kMaxExp || nn < 0 || nn > kMaxExp || oo < 0 || oo > kMaxExp) {
                *status = CUTC_ERR_INVALID;
                continue;
            }
            const double cc = c[k];
            if (!(fabs(cc) >= 1e-10))
                continue;
            if (nt >= kMaxTerms) {
                *status = CUTC_ERR_INVALID;
                continue;
            }
            coef[3 * nt] = cc * mm;
            coef[3 * nt + 1] = cc * nn;
            coef[3 * nt + 2] = cc * oo;
            exps[nt] = mm | (nn << 3) | (oo << 6);
            nt++;
        }
    }
    off[nN] = nt;
}

// Device address of the scratch, looked up once per device with that device
// current (the host-side name of a __device__ array is only a stand-in).
static int noalloc_scratch(unsigned char **out)
{
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static unsigned char *addr[kMaxDevices] = {};
    int dev = 0;
    CUTC_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        cutc_set_error(CUTC_ERR_NO_DEVICE, "device ordinal %d out of range", dev);
        return CUTC_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            cutc_set_error(CUTC_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
            return CUTC_ERR_CUDA;
        }
        addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = addr[dev];
    return CUTC_OK;
}

}  // namespace cutc

extern "C" int cutc_jast_bh_dev_noalloc(int i0, int n1b, int n_grid1, int n_grid2, int n_nuc,
                                        int size_bh, const double *r1, const double *r2,
                                        const double *rn, const double *c_bh, const int *m_bh,
                                        const int *n_bh, const int *o_bh, double a_en, double a_ee,
                                        double *grad1u, void *stream)
{
    using namespace cutc;
    if (n1b <= 0 || n_grid2 <= 0 || n_nuc <= 0 || size_bh < 0 || i0 < 0 || i0 + n1b > n_grid1 ||
        n_nuc > kMaxNuc || !r1 || !r2 || !rn || !grad1u || !(a_en > 0) || !(a_ee > 0) ||
        (size_bh > 0 && (!c_bh || !m_bh || !n_bh || !o_bh))) {
        cutc_set_error(CUTC_ERR_INVALID, "invalid pair-kernel arguments");
        return CUTC_ERR_INVALID;
    }
    const size_t need = kNaT1 + (size_t)n1b * n_nuc * sizeof(NucTerm) +
                        (size_t)n_nuc * n_grid2 * sizeof(double) + 256;
    if (need > kNoAllocScratchBytes) {
        cutc_set_error(CUTC_ERR_INVALID,
                       "%zu bytes of scratch needed (n1b=%d, n_grid2=%d, n_nuc=%d) exceed the "
                       "%zu-byte static scratch of the allocation-free entry point",
                       need, n1b, n_grid2, n_nuc, kNoAllocScratchBytes);
        return CUTC_ERR_INVALID;
    }
    unsigned char *base = nullptr;
    CUTC_TRY(noalloc_scratch(&base));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int *status = reinterpret_cast<int *>(base + kNaStatus);
    double *coef = reinterpret_cast<double *>(base + kNaCoef);
    int *exps = reinterpret_cast<int *>(base + kNaExps);
    int *off = reinterpret_cast<int *>(base + kNaOff);
    NucTerm *t1 = reinterpret_cast<NucTerm *>(base + kNaT1);
    const size_t t1_bytes = ((size_t)n1b * n_nuc * sizeof(NucTerm) + 255) & ~(size_t)255;
    double *f2 = reinterpret_cast<double *>(base + kNaT1 + t1_bytes);

    // the scratch keeps the previous call's contents: only the status must start at zero
    CUTC_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
    noalloc_terms_kernel<<<1, 1, 0, st>>>(n_nuc, size_bh, c_bh, m_bh, n_bh, o_bh, coef, exps, off,
                                          status);
    CUTC_CUDA_TRY(cudaGetLastError());
    CUTC_TRY(launch_r1_terms(st, i0, n1b, n_nuc, r1, rn, a_en, t1));
    CUTC_TRY(launch_r2_terms(st, n_grid2, n_nuc, r2, rn, a_en, f2));
    PairArgs P;
    P.i0 = i0; P.n1b = n1b; P.n2 = n_grid2; P.nN = n_nuc;
    // the kernel reads the term count from off[nN]; size its shared memory for the maximum
    P.n_terms = (int)std::min<int64_t>(kMaxTerms, (int64_t)n_nuc * size_bh);
    P.r1 = r1; P.r2 = r2; P.t1 = t1; P.f2 = f2;
    P.coef = coef; P.exps = exps; P.term_off = off; P.a_ee = a_ee;
    P.G = grad1u; P.ldg = n_grid2; P.plane = (int64_t)n1b * n_grid2;
    CUTC_TRY(launch_pair_f64(st, P));
    note_launches(4);
    int h_status = 0;
    CUTC_CUDA_TRY(cudaMemcpyAsync(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUTC_CUDA_TRY(cudaStreamSynchronize(st));
    if (h_status != CUTC_OK) {
        cutc_set_error(h_status, "Jastrow exponent outside [0, %d] or more than %d terms", kMaxExp,
                       kMaxTerms);
        return h_status;
    }
    return CUTC_OK;
}
