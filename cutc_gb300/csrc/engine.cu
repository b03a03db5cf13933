// Host orchestration of one integral build on one GPU (sm_103a).
//
// Counterpart of the reference's host drivers src/cutc_int.c:15-243,
// src/build_int2_grad1_u12_ao.cu:9-347 and src/build_int_2e_ao.cu:11-145,
// redesigned:
//   * one engine per device with its own streams and a
//     grow-only workspace (no cudaMalloc/cudaFree per call, no
//     cudaDeviceSynchronize between steps: everything is stream-ordered);
//   * r1 is tiled by a byte budget in 64-bit arithmetic (the reference sizes
//     tiles in 32-bit int and from bytes instead of doubles);
//   * the AO-pair products are packed (symmetric / antisymmetric halves), so
//     both contractions do half (X) and a quarter (int_2e) of the dense work;
//   * X is accumulated per r1 tile with beta = 0, so r1 tiling is exact (the
//     reference keeps beta = 1 across r1 passes, src/build_int2_grad1_u12_ao.cu:166);
//   * errors are returned as status codes, never exit().
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "aos.cuh"
#include "common.cuh"
#include "dgemm.cuh"
#include "engine.cuh"
#include "pair.cuh"
#include "products.cuh"
#include "split.cuh"

static thread_local char g_err[512] = "";

void cutc_set_error(int status, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    int n = snprintf(g_err, sizeof(g_err), "[status %d] ", status);
    if (n < 0)
        n = 0;
    vsnprintf(g_err + n, sizeof(g_err) - (size_t)n, fmt, ap);
    va_end(ap);
}

extern "C" const char *cutc_last_error(void) { return g_err; }

namespace cutc {

static std::atomic<long> g_launches{0};
void note_launches(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long launches_so_far() { return g_launches.load(std::memory_order_relaxed); }

// ---------------------------------------------------------------------------
// engine and workspace
// ---------------------------------------------------------------------------

int Workspace::get(int slot, size_t bytes, void **out)
{
    if (slot >= (int)bufs.size())
        bufs.resize(slot + 1);
    Buf &b = bufs[slot];
    bytes = (bytes + 255) & ~(size_t)255;
    if (bytes == 0)
        bytes = 256;
    if (b.cap < bytes) {
        if (b.p) {
            cudaFree(b.p);
            b.p = nullptr;
            b.cap = 0;
        }
        cudaError_t e = cudaMalloc(&b.p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            cutc_set_error(CUTC_ERR_NO_MEMORY, "cudaMalloc(%zu) for workspace slot %d: %s", bytes,
                           slot, cudaGetErrorString(e));
            return CUTC_ERR_NO_MEMORY;
        }
        b.cap = bytes;
    }
    *out = b.p;
    return CUTC_OK;
}

int PinnedPool::get(int k, size_t bytes, void **out)
{
    Buf &b = bufs[k];
    bytes = std::max<size_t>(4096, (bytes + 4095) & ~(size_t)4095);
    if (b.cap < bytes) {
        if (b.p) {
            cudaFreeHost(b.p);
            b.p = nullptr;
            b.cap = 0;
        }
        cudaError_t e = cudaHostAlloc(&b.p, bytes, cudaHostAllocDefault);
        if (e != cudaSuccess) {
            cudaGetLastError();
            b.p = nullptr;
            cutc_set_error(CUTC_ERR_NO_MEMORY, "cudaHostAlloc(%zu) for output staging: %s", bytes,
                           cudaGetErrorString(e));
            return CUTC_ERR_NO_MEMORY;
        }
        b.cap = bytes;
    }
    *out = b.p;
    return CUTC_OK;
}

void PinnedPool::release()
{
    for (auto &b : bufs) {
        if (b.p)
            cudaFreeHost(b.p);
        b.p = nullptr;
        b.cap = 0;
    }
}

// Host copy split over a few threads (page faults of fresh caller memory and
// the copy itself both scale with threads).
static void host_copy(void *dst, const void *src, size_t bytes)
{
    // first-touch page faults of fresh caller memory dominate large copies and
    // scale with threads: up to half the host's cores
    const size_t kChunk = (size_t)16 << 20;
    static const int kMaxThreads =
        (int)std::max(2u, std::min(8u, std::thread::hardware_concurrency() / 2));
    const int n = (int)std::min<size_t>(kMaxThreads, bytes / kChunk);
    if (n <= 1) {
        memcpy(dst, src, bytes);
        return;
    }
    const size_t per = ((bytes + n - 1) / n + 4095) & ~(size_t)4095;
    std::vector<std::thread> th;
    for (int k = 1; k < n; k++) {
        const size_t o = (size_t)k * per;
        if (o >= bytes)
            break;
        th.emplace_back([=] { memcpy((char *)dst + o, (const char *)src + o, std::min(per, bytes - o)); });
    }
    memcpy(dst, src, std::min(per, bytes));
    for (auto &t : th)
        t.join();
}

// True when the device can copy into p asynchronously (pinned, registered or managed).
static bool async_host_ptr(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged;
}

void Workspace::release()
{
    for (auto &b : bufs)
        if (b.p)
            cudaFree(b.p);
    bufs.clear();
    std::lock_guard<std::mutex> lk(memo_mu);
    memo = PlanMemo{};
}

bool Workspace::recall(uint64_t key, PlanMemo *out)
{
    std::lock_guard<std::mutex> lk(memo_mu);
    if (memo.key == 0 || memo.key != key)
        return false;
    *out = memo;
    return true;
}

void Workspace::remember(const PlanMemo &m)
{
    std::lock_guard<std::mutex> lk(memo_mu);
    memo = m;
}

static std::mutex g_engines_mu;
static std::vector<Engine *> g_engines;

// The remembered default plan of the current device's engine for a build of shape
// `key` (false without an engine or a plan of that shape).
static bool engine_recall(uint64_t key, PlanMemo *out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    std::lock_guard<std::mutex> lk(g_engines_mu);
    return dev < (int)g_engines.size() && g_engines[dev] && g_engines[dev]->ws.recall(key, out);
}

int make_engine(int dev, Engine **out)
{
    cudaDeviceProp prop;
    CUTC_CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
    if (prop.major != 10 || prop.minor != 3) {
        cutc_set_error(CUTC_ERR_NO_DEVICE,
                       "device %d is sm_%d%d; this library is built for sm_103a (GB300)", dev,
                       prop.major, prop.minor);
        return CUTC_ERR_NO_DEVICE;
    }
    Engine *E = new Engine();
    E->device = dev;
    E->n_sm = prop.multiProcessorCount;
    E->max_threads_per_block = prop.maxThreadsPerBlock;
    for (int k = 0; k < 3; k++)
        E->max_grid[k] = prop.maxGridSize[k];
    cudaError_t e = cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&E->xfer, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        for (int k = 0; k < kNumEvents && e == cudaSuccess; k++)
            e = cudaEventCreate(&E->ev[k]);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cutc_set_error(CUTC_ERR_CUDA, "engine setup: %s", cudaGetErrorString(e));
        delete E;
        return CUTC_ERR_CUDA;
    }
    *out = E;
    return CUTC_OK;
}

void destroy_engine(Engine *E)
{
    if (!E)
        return;
    cudaStreamSynchronize(E->stream);
    cudaStreamSynchronize(E->xfer);
    E->ws.release();
    E->pinned.release();
    for (auto e : E->tile_ev)
        cudaEventDestroy(e);
    for (int k = 0; k < kNumEvents; k++)
        cudaEventDestroy(E->ev[k]);
    cudaStreamSynchronize(E->xfer);
    cudaStreamDestroy(E->xfer);
    cudaStreamDestroy(E->stream);
    delete E;
}

int get_engine(Engine **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cutc_set_error(CUTC_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
        return CUTC_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lk(g_engines_mu);
    if ((int)g_engines.size() <= dev)
        g_engines.resize(dev + 1, nullptr);
    if (!g_engines[dev])
        CUTC_TRY(make_engine(dev, &g_engines[dev]));
    *out = g_engines[dev];
    return CUTC_OK;
}

// ---------------------------------------------------------------------------
// request preparation
// ---------------------------------------------------------------------------

int build_terms(const Request &R, std::vector<double> &coef, std::vector<int> &exps,
                std::vector<int> &off)
{
    coef.clear();
    exps.clear();
    off.assign(R.nN + 1, 0);
    for (int A = 0; A < R.nN; A++) {
        off[A] = (int)exps.size();
        for (int p = 0; p < R.nB; p++) {
            const int k = p + R.nB * A;  // Fortran (size_bh, n_nuc)
            const int m = R.m_bh[k], n = R.n_bh[k], o = R.o_bh[k];
            if (m < 0 || m > kMaxExp || n < 0 || n > kMaxExp || o < 0 || o > kMaxExp) {
                cutc_set_error(CUTC_ERR_INVALID,
                               "Jastrow exponent out of [0, %d] at term %d of nucleus %d "
                               "(m=%d n=%d o=%d)", kMaxExp, p, A, m, n, o);
                return CUTC_ERR_INVALID;
            }
            const double c = R.c_bh[k];
            if (!(std::fabs(c) >= 1e-10))  // skipped like src/jast_bh.cu:203 (NaN skipped too)
                continue;
            coef.push_back(c * m);
            coef.push_back(c * n);
            coef.push_back(c * o);
            exps.push_back(m | (n << 3) | (o << 6));
        }
    }
    off[R.nN] = (int)exps.size();
    if ((int)exps.size() > kMaxTerms) {
        cutc_set_error(CUTC_ERR_INVALID, "%d Jastrow terms exceed the limit %d", (int)exps.size(),
                       kMaxTerms);
        return CUTC_ERR_INVALID;
    }
    return CUTC_OK;
}

static int validate(const Request &R)
{
    if (R.n1 <= 0 || R.n2 <= 0 || R.nA <= 0 || R.nN <= 0 || R.nB < 0) {
        cutc_set_error(CUTC_ERR_INVALID, "sizes must be positive (n_grid1=%d n_grid2=%d n_ao=%d "
                       "n_nuc=%d size_bh=%d)", R.n1, R.n2, R.nA, R.nN, R.nB);
        return CUTC_ERR_INVALID;
    }
    if (R.nN > kMaxNuc) {
        cutc_set_error(CUTC_ERR_INVALID, "n_nuc=%d exceeds %d", R.nN, kMaxNuc);
        return CUTC_ERR_INVALID;
    }
    if ((int64_t)R.nA * R.nA > (int64_t)INT32_MAX / 2) {
        cutc_set_error(CUTC_ERR_INVALID, "n_ao=%d too large", R.nA);
        return CUTC_ERR_INVALID;
    }
    if (R.x_only && R.i_only) {
        cutc_set_error(CUTC_ERR_INVALID, "NULL X and int_2e outputs: nothing to build");
        return CUTC_ERR_INVALID;
    }
    const void *ptrs[] = {R.r1, R.r2, R.wr2, R.rn, R.i_only ? R.I : R.X,
                          R.x_only ? R.X : R.wr1, R.x_only ? R.X : R.I};
    for (const void *p : ptrs)
        if (!p) {
            cutc_set_error(CUTC_ERR_INVALID, "NULL array argument");
            return CUTC_ERR_INVALID;
        }
    if ((!R.aos1 && !R.x_only) || !R.aos2) {
        if (!R.basis) {
            cutc_set_error(CUTC_ERR_INVALID, "NULL AO array and no basis to evaluate it from");
            return CUTC_ERR_INVALID;
        }
        CUTC_TRY(validate_basis(R.basis, R.nA));
    }
    if (R.nB > 0 && (!R.c_bh || !R.m_bh || !R.n_bh || !R.o_bh)) {
        cutc_set_error(CUTC_ERR_INVALID, "NULL Jastrow parameter array");
        return CUTC_ERR_INVALID;
    }
    if (!(R.a_en > 0.0) || !(R.a_ee > 0.0)) {
        cutc_set_error(CUTC_ERR_INVALID, "a_en and a_ee must be positive");
        return CUTC_ERR_INVALID;
    }
    if (R.x_components != 3 && R.x_components != 4) {
        cutc_set_error(CUTC_ERR_INVALID, "x_components must be 3 or 4");
        return CUTC_ERR_INVALID;
    }
    if (R.precision != CUTC_PLAIN_FP64 && R.precision != CUTC_SPLIT_BF16) {
        cutc_set_error(CUTC_ERR_INVALID, "unknown precision form %d", R.precision);
        return CUTC_ERR_INVALID;
    }
    if (R.int2e_layout != CUTC_INT2E_PQST && R.int2e_layout != CUTC_INT2E_PSQT) {
        cutc_set_error(CUTC_ERR_INVALID, "unknown int_2e layout %d", R.int2e_layout);
        return CUTC_ERR_INVALID;
    }
    if (R.k_split < 0 || (R.k_split > 0 && R.k_split < 64)) {
        cutc_set_error(CUTC_ERR_INVALID, "k_split must be 0 or at least 64");
        return CUTC_ERR_INVALID;
    }
    if (R.precision == CUTC_SPLIT_BF16 && (R.n_slices < 3 || R.n_slices > kMaxSlices)) {
        cutc_set_error(CUTC_ERR_INVALID, "n_slices must be in [3, %d]", kMaxSlices);
        return CUTC_ERR_INVALID;
    }
    return CUTC_OK;
}

// ---------------------------------------------------------------------------
// the build
// ---------------------------------------------------------------------------

enum Slot {
    S_R1, S_WR1, S_R2, S_WR2, S_RN, S_AOS1, S_AOS2, S_COEF, S_EXPS, S_OFF,
    S_T1, S_F2, S_P, S_G, S_XP, S_S0, S_SL, S_H, S_N, S_XOUT, S_XOUT1, S_IOUT, S_IOUT1,
    S_R2D, S_F2D, S_POLY, S_BASIS,
    S_SPLIT0  // split-form slots follow
};

static inline double ev_ms(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

// Columns of int_2e per output slab when int_2e goes to the host: a slab is
// assembled on the device and copied out while the next one is assembled.  A
// slab is a whole number of the slowest index t (nA columns), so it is one
// contiguous block in both int_2e layouts.
// CUTC_INT2E_SLAB_COLS overrides the 1 GiB slab (rounded down to nA columns).
static int int2e_slab_cols(int nA)
{
    const int64_t n = (int64_t)nA * nA;
    int64_t per = ((int64_t)1 << 30) / (n * 8);
    if (const char *e = getenv("CUTC_INT2E_SLAB_COLS"))
        per = atoll(e);
    per = per / nA * nA;
    return (int)std::min<int64_t>(n, std::max<int64_t>(nA, per));
}

// Device bytes of a build that do not grow with the r1 tile (besides the
// molecule arrays): r2 terms, the P operand, H and N, int_2e output slabs.
static size_t fixed_bytes(const Request &R)
{
    const int64_t n2 = R.n2, nA = R.nA, nN = R.nN;
    const int64_t np = n_pairs(nA), nl = std::max<int64_t>(1, n_strict_pairs(nA));
    double b = (double)nN * n2 * 8;
    if (!R.x_only)
        b += ((double)np * np + (double)np * nl) * 8;
    if (R.precision == CUTC_PLAIN_FP64)
        b += (double)np * n2 * 8;
    else
        b += (double)split_fixed_bytes(R) + (3.0 + nN) * n2 * sizeof(float2) +
             (double)split_pair_fixed_bytes(R);
    if (!(R.device_pointers || R.out_device) && !R.x_only)
        b += 2.0 * int2e_slab_cols(R.nA) * nA * nA * 8;
    return (size_t)b;
}

// Device bytes per r1 row of an X tile: G, per-point terms, output staging (two
// buffers) and, split form, G's slices and polynomial coefficients.
static size_t r1_row_bytes(const Request &R)
{
    size_t b = 4 * (size_t)R.n2 * 8 + (size_t)R.nN * sizeof(NucTerm);
    if (!(R.device_pointers || R.out_device) && !R.i_only)
        b += 2 * (size_t)R.x_components * R.nA * R.nA * 8;
    if (R.precision == CUTC_SPLIT_BF16)
        b += split_r1_row_bytes(R) + pair_df_poly_bytes(6, 1, R.nN) + split_pair_row_bytes(R);
    return b;
}

// Device bytes per r1 row of an int_2e block: the packed X rows and the block's
// r1 operands of the int_2e contractions.
static size_t int2e_row_bytes(const Request &R)
{
    const int64_t np = n_pairs(R.nA), nl = std::max<int64_t>(1, n_strict_pairs(R.nA));
    size_t b = 4 * (size_t)np * 8;
    if (R.x_only)  // the packed X rows alone, staged for the expansion
        return b;
    if (R.precision == CUTC_PLAIN_FP64)
        b += ((size_t)np + 3 * (size_t)nl) * 8;
    else
        b += split_int2e_row_bytes(R);
    return b;
}

// The shape of a build as far as the sizes of its working buffers go (FNV-1a over the
// fields that set them; never 0).
static uint64_t plan_key(const Request &R)
{
    const int64_t f[] = {R.n1, R.n2, R.nA, R.nN, R.precision, R.n_slices, R.x_components,
                         (R.device_pointers || R.out_device) ? 1 : 0, R.x_only, R.i_only,
                         R.tile_rows, R.int2e_rows};
    uint64_t h = 1469598103934665603ull;
    for (int64_t v : f)
        for (int k = 0; k < 8; k++) {
            h ^= (uint64_t)(v >> (8 * k)) & 0xffu;
            h *= 1099511628211ull;
        }
    return h ? h : 1;
}

// r1 rows per X tile and per int_2e block for a budget (each gets the budget): the
// int_2e contractions run once per block, with K = its rows, so the block is made
// as large as its budget allows and cut into equal X tiles that each fit theirs.
// CUTC_TILE_ROWS / CUTC_INT2E_ROWS cap them.  A tile has at most kMaxTileRows rows:
// the pair kernels give each CTA at most 8 r1 rows along gridDim.y (<= 65535).
constexpr int64_t kMaxTileRows = (int64_t)1 << 18;

static void plan_rows(const Request &R, size_t budget, int64_t *n1t, int64_t *kb)
{
    const int64_t n1 = R.n1;
    int64_t t = std::max<int64_t>(1, std::min<int64_t>((int64_t)(budget / r1_row_bytes(R)), n1));
    t = std::min(t, kMaxTileRows);
    if (R.tile_rows > 0)
        t = std::min<int64_t>(t, R.tile_rows);
    if (R.x_only) {  // no int_2e: the block is the tile
        *n1t = t;
        *kb = t;
        return;
    }
    int64_t k = std::max<int64_t>(1, std::min<int64_t>((int64_t)(budget / int2e_row_bytes(R)), n1));
    if (R.int2e_rows > 0)
        k = std::min<int64_t>(k, R.int2e_rows);
    const int64_t per = (k + t - 1) / t;  // tiles per block
    if (k >= n1) {
        *kb = n1;
        *n1t = (n1 + per - 1) / per;
    } else {
        *n1t = k / per;
        *kb = per * *n1t;
    }
}

size_t build_footprint(const Request &R, size_t tile_budget)
{
    const int64_t n1 = R.n1, n2 = R.n2, nA = R.nA, nN = R.nN;
    int64_t n1t, kb;
    plan_rows(R, tile_budget, &n1t, &kb);
    double b = (double)fixed_bytes(R) + (double)n1t * r1_row_bytes(R) +
               (double)kb * int2e_row_bytes(R);
    if (!(R.device_pointers || R.in_device))
        b += (4.0 * n1 + 4.0 * n2 + 3.0 * nN + 4.0 * n1 * nA + (double)n2 * nA) * 8;
    return (size_t)(b * 1.05) + ((size_t)64 << 20);
}

// Waits for the build's copies and kernels on every exit path, so that no copy
// into the caller's arrays is still running when the call returns.
struct StreamsDrain {
    cudaStream_t a, b;
    ~StreamsDrain()
    {
        cudaStreamSynchronize(b);
        cudaStreamSynchronize(a);
    }
};

int run_build(Engine *E, const Request &R_in, cutc_stats *stats)
{
    CUTC_TRY(validate(R_in));
    Request R = R_in;
    // The term table is built on the host; with device pointers the Jastrow
    // parameters are brought over first (they are tiny: size_bh x n_nuc).
    std::vector<double> h_c;
    std::vector<int> h_m, h_n, h_o;
    if (R.device_pointers && R.nB > 0) {  // Jastrow parameters on the device
        const size_t nt_in = (size_t)R.nB * R.nN;
        cudaStream_t s0 = R.stream ? R.stream : E->stream;
        h_c.resize(nt_in);
        h_m.resize(nt_in);
        h_n.resize(nt_in);
        h_o.resize(nt_in);
        CUTC_CUDA_TRY(cudaMemcpyAsync(h_c.data(), R.c_bh, nt_in * 8, cudaMemcpyDeviceToHost, s0));
        CUTC_CUDA_TRY(cudaMemcpyAsync(h_m.data(), R.m_bh, nt_in * 4, cudaMemcpyDeviceToHost, s0));
        CUTC_CUDA_TRY(cudaMemcpyAsync(h_n.data(), R.n_bh, nt_in * 4, cudaMemcpyDeviceToHost, s0));
        CUTC_CUDA_TRY(cudaMemcpyAsync(h_o.data(), R.o_bh, nt_in * 4, cudaMemcpyDeviceToHost, s0));
        CUTC_CUDA_TRY(cudaStreamSynchronize(s0));
        R.c_bh = h_c.data();
        R.m_bh = h_m.data();
        R.n_bh = h_n.data();
        R.o_bh = h_o.data();
    }
    std::vector<double> coef;
    std::vector<int> exps, off;
    CUTC_TRY(build_terms(R, coef, exps, off));

    cudaStream_t st = R.stream ? R.stream : E->stream;
    Workspace &W = E->ws;
    const int n1 = R.n1, n2 = R.n2, nA = R.nA, nN = R.nN;
    const int64_t np = n_pairs(nA), nl = n_strict_pairs(nA), nA2 = (int64_t)nA * nA;
    const long launches0 = launches_so_far();

    CUTC_CUDA_TRY(cudaEventRecord(E->ev[0], st));

    // ---- inputs on the device --------------------------------------------
    const double *d_r1 = nullptr, *d_wr1 = nullptr, *d_r2 = nullptr, *d_wr2 = nullptr;
    const double *d_rn = nullptr, *d_aos1 = nullptr, *d_aos2v = nullptr;
    bool aos1_deferred = false;
    void *p;
    auto put = [&](int slot, const void *h, size_t bytes, const double **dst) -> int {
        CUTC_TRY(W.get(slot, bytes, &p));
        CUTC_CUDA_TRY(cudaMemcpyAsync(p, h, bytes, cudaMemcpyHostToDevice, st));
        *dst = (const double *)p;
        return CUTC_OK;
    };
    const bool in_dev = R.device_pointers || R.in_device;
    const bool out_dev = R.device_pointers || R.out_device;
    if (in_dev) {
        d_r1 = R.r1; d_wr1 = R.wr1; d_r2 = R.r2; d_wr2 = R.wr2; d_rn = R.rn;
        d_aos1 = R.aos1;
        d_aos2v = R.aos2;  // component 0 is the first n2*nA block
    } else {
        CUTC_TRY(put(S_R1, R.r1, 3 * (size_t)n1 * 8, &d_r1));
        if (R.wr1)
            CUTC_TRY(put(S_WR1, R.wr1, (size_t)n1 * 8, &d_wr1));
        CUTC_TRY(put(S_R2, R.r2, 3 * (size_t)n2 * 8, &d_r2));
        CUTC_TRY(put(S_WR2, R.wr2, (size_t)n2 * 8, &d_wr2));
        CUTC_TRY(put(S_RN, R.rn, 3 * (size_t)nN * 8, &d_rn));
        if (R.aos1 && !R.x_only) {
            // the AO values on r1, the largest input, are read only by the int_2e blocks:
            // they are copied on the transfer stream once the first tile is queued
            CUTC_TRY(W.get(S_AOS1, 4 * (size_t)n1 * nA * 8, &p));
            d_aos1 = (const double *)p;
            aos1_deferred = true;
        }
        // only the value component of aos_data2 is used (src/long_range_integ.cu:30-35)
        if (R.aos2)
            CUTC_TRY(put(S_AOS2, R.aos2, (size_t)n2 * nA * 8, &d_aos2v));
    }
    if ((!R.aos1 && !R.x_only) || !R.aos2) {
        // AO values (and r1 gradients) from the basis, on the device
        BasisDev B;
        CUTC_TRY(upload_basis(W, S_BASIS, st, R.basis, &B));
        if (!R.aos1 && !R.x_only) {
            CUTC_TRY(W.get(S_AOS1, 4 * (size_t)n1 * nA * 8, &p));
            CUTC_TRY(launch_eval_aos(st, B, n1, d_r1, 4, (double *)p, n1));
            d_aos1 = (const double *)p;
        }
        if (!R.aos2) {
            CUTC_TRY(W.get(S_AOS2, (size_t)n2 * nA * 8, &p));
            CUTC_TRY(launch_eval_aos(st, B, n2, d_r2, 1, (double *)p, n2));
            d_aos2v = (const double *)p;
        }
    }
    // leading dimension of the AO values on r1 on the device: a window of a caller's
    // device array keeps the caller's stride; uploaded or evaluated arrays are packed
    const int64_t ld_a1 = (in_dev && R.aos1 && R.ld1 > 0) ? R.ld1 : n1;
    const int nt = (int)exps.size();
    double *d_coef;
    int *d_exps, *d_off;
    CUTC_TRY(W.get(S_COEF, std::max<size_t>(1, coef.size()) * 8, &p));
    d_coef = (double *)p;
    CUTC_TRY(W.get(S_EXPS, std::max<size_t>(1, exps.size()) * 4, &p));
    d_exps = (int *)p;
    CUTC_TRY(W.get(S_OFF, off.size() * 4, &p));
    d_off = (int *)p;
    if (nt) {
        CUTC_CUDA_TRY(cudaMemcpyAsync(d_coef, coef.data(), coef.size() * 8, cudaMemcpyHostToDevice, st));
        CUTC_CUDA_TRY(cudaMemcpyAsync(d_exps, exps.data(), exps.size() * 4, cudaMemcpyHostToDevice, st));
    }
    CUTC_CUDA_TRY(cudaMemcpyAsync(d_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice, st));
    CUTC_CUDA_TRY(cudaEventRecord(E->ev[1], st));

    // ---- r1 tiling ---------------------------------------------------------
    // Every r1 tile is carried all the way: pair terms, then its X rows, written
    // out and kept in the int_2e block buffer.  When a block of whole tiles is
    // complete, its share of the int_2e contractions (K = its rows) is added to H
    // and N in FP64.  Device memory is the fixed part plus one tile and one block,
    // each within the budget.
    size_t budget = R.max_work_bytes;
    int64_t n1t, kb;
    PlanMemo memo;
    const uint64_t key = plan_key(R);
    // which pair-term buffers the build holds besides: the remembered plan is taken
    // only when they are the same
    uint64_t path = 1 + (R.pair_fp64 ? 2 : 0);
    if (R.precision == CUTC_SPLIT_BF16 && !R.pair_fp64)
        path += 4 * (uint64_t)split_pair_tc_ok(R, exps.data(), nt) +
                8 * (uint64_t)pair_df_max_exp(exps.data(), nt);
    const bool default_budget = budget == 0;
    if (default_budget && E->ws.recall(key, &memo) && memo.path == path) {
        budget = memo.budget;  // the last build of this shape: its buffers fit this plan
        n1t = memo.n1t;
        kb = memo.kb;
    } else {
        if (default_budget) {
            size_t free_b = 0, total_b = 0;
            CUTC_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
            budget = std::min<size_t>((size_t)24 << 30, free_b / 4);
            const size_t fixed = fixed_bytes(R);
            if (free_b > fixed)
                budget = std::min<size_t>(budget, (size_t)((double)(free_b - fixed) * 0.4));
        }
        plan_rows(R, budget, &n1t, &kb);
    }
    const int n_tiles = (int)((n1 + n1t - 1) / n1t);
    constexpr int kTileEv = 6;
    if (stats) {
        while ((int)E->tile_ev.size() < kTileEv * n_tiles) {
            cudaEvent_t e;
            CUTC_CUDA_TRY(cudaEventCreate(&e));
            E->tile_ev.push_back(e);
        }
    }

    // ---- buffers -------------------------------------------------------------
    NucTerm *d_t1;
    double *d_f2, *d_P = nullptr, *d_G, *d_Xt, *d_H = nullptr, *d_N = nullptr;
    double *d_S0 = nullptr, *d_Sl = nullptr;
    double *stage_x[2] = {nullptr, nullptr}, *stage_i[2] = {nullptr, nullptr};
    CUTC_TRY(W.get(S_T1, (size_t)n1t * nN * sizeof(NucTerm), &p));
    d_t1 = (NucTerm *)p;
    CUTC_TRY(W.get(S_F2, (size_t)nN * n2 * 8, &p));
    d_f2 = (double *)p;
    CUTC_TRY(W.get(S_G, 4 * (size_t)n1t * n2 * 8, &p));
    d_G = (double *)p;
    CUTC_TRY(W.get(S_XP, 4 * (size_t)kb * np * 8, &p));
    d_Xt = (double *)p;  // the int_2e block: Xt[(m blk_rows + i) np + p]
    if (!R.x_only) {
        CUTC_TRY(W.get(S_H, (size_t)np * np * 8, &p));
        d_H = (double *)p;
        CUTC_TRY(W.get(S_N, (size_t)np * std::max<int64_t>(nl, 1) * 8, &p));
        d_N = (double *)p;
    }
    const int slab = int2e_slab_cols(nA);
    if (!out_dev) {
        for (int k = 0; k < 2; k++) {
            if (!R.i_only) {
                CUTC_TRY(W.get(S_XOUT + k, (size_t)R.x_components * n1t * nA2 * 8, &p));
                stage_x[k] = (double *)p;
            }
            if (!R.x_only) {
                CUTC_TRY(W.get(S_IOUT + k, (size_t)slab * nA2 * 8, &p));
                stage_i[k] = (double *)p;
            }
        }
    }
    if (R.precision == CUTC_PLAIN_FP64 && !R.x_only) {
        CUTC_TRY(W.get(S_S0, (size_t)np * kb * 8, &p));
        d_S0 = (double *)p;
        CUTC_TRY(W.get(S_SL, (size_t)std::max<int64_t>(nl, 1) * 3 * kb * 8, &p));
        d_Sl = (double *)p;
    }
    CUTC_TRY(launch_r2_terms(st, n2, nN, d_r2, d_rn, R.a_en, d_f2));
    note_launches(1);

    SplitPlan sp;
    float2 *d_r2d = nullptr, *d_f2d = nullptr, *d_poly = nullptr;
    int pexp = 4;
    bool psparse = false;
    if (R.precision == CUTC_SPLIT_BF16) {
        pexp = pair_df_max_exp(exps.data(), nt);
        psparse = pexp == 4 && pair_df_sparse(exps.data(), nt) && !getenv("CUTC_PAIR_DENSE");
        CUTC_TRY(W.get(S_R2D, 3 * (size_t)n2 * sizeof(float2), &p));
        d_r2d = (float2 *)p;
        CUTC_TRY(W.get(S_F2D, (size_t)nN * n2 * sizeof(float2), &p));
        d_f2d = (float2 *)p;
        CUTC_TRY(W.get(S_POLY, pair_df_poly_bytes(pexp, (int)n1t, nN), &p));
        d_poly = (float2 *)p;
        CUTC_TRY(launch_r2_df(st, n2, nN, d_r2, d_f2, d_r2d, d_f2d));
        note_launches(1);
    }
    if (R.precision == CUTC_PLAIN_FP64) {
        CUTC_TRY(W.get(S_P, (size_t)np * n2 * 8, &p));
        d_P = (double *)p;
        if (!(R.mol_tag && E->tag_x == R.mol_tag && E->tag_x_buf == d_P)) {
            CUTC_TRY(launch_sym_products(st, n2, nA, d_wr2, d_aos2v, n2, d_P, n2));
            note_launches(1);
            E->tag_x = R.mol_tag;
            E->tag_x_buf = d_P;
        }
    } else {
        CUTC_TRY(split_prepare_x(E, R, st, d_wr2, d_aos2v, n1t, S_SPLIT0, sp));
        if (split_pair_tc_ok(R, exps.data(), nt))
            CUTC_TRY(split_pair_prepare(E, R, st, d_f2, n1t, sp));
    }
    CUTC_CUDA_TRY(cudaEventRecord(E->ev[2], st));

    // ---- tiles ---------------------------------------------------------------
    // Host outputs leave through two device staging buffers, copied on the
    // transfer stream while the next tile computes.  Pinned (or managed) caller
    // memory takes the copies directly; pageable caller memory gets them in two
    // pinned buffers first, from which this thread copies while the device
    // works on (no pageable cudaMemcpy, which holds the thread until the stream
    // reaches it).
    StreamsDrain drain{st, E->xfer};
    cudaEvent_t ready[2] = {E->ev[3], E->ev[4]}, done[2] = {E->ev[9], E->ev[10]};
    bool busy[2] = {false, false};
    const bool x_direct = out_dev || R.i_only || async_host_ptr(R.X);
    const bool i_direct = out_dev || R.x_only || async_host_ptr(R.I);
    double *hpin_x[2] = {nullptr, nullptr}, *hpin_i[2] = {nullptr, nullptr};
    for (int k = 0; k < 2 && !out_dev; k++) {
        if (!x_direct) {
            CUTC_TRY(E->pinned.get(k, (size_t)R.x_components * n1t * nA2 * 8, &p));
            hpin_x[k] = (double *)p;
        }
        if (!i_direct) {
            CUTC_TRY(E->pinned.get(2 + k, (size_t)slab * nA2 * 8, &p));
            hpin_i[k] = (double *)p;
        }
    }
    auto tile_rows = [&](int tile, int64_t *i0, int64_t *nb) {
        *i0 = (int64_t)tile * n1t;
        *nb = std::min<int64_t>(n1t, n1 - *i0);
    };
    auto copy_x = [&](int tile) -> int {  // device staging -> caller memory or pinned
        const int b = tile & 1;
        int64_t i0, nb;
        tile_rows(tile, &i0, &nb);
        CUTC_CUDA_TRY(cudaStreamWaitEvent(E->xfer, ready[b], 0));
        if (x_direct) {
            for (int m = 0; m < R.x_components; m++)
                CUTC_CUDA_TRY(cudaMemcpyAsync(R.X + ((int64_t)m * n1 + i0) * nA2,
                                              stage_x[b] + (int64_t)m * nb * nA2,
                                              (size_t)nb * nA2 * 8, cudaMemcpyDeviceToHost, E->xfer));
        } else {
            CUTC_CUDA_TRY(cudaMemcpyAsync(hpin_x[b], stage_x[b],
                                          (size_t)R.x_components * nb * nA2 * 8,
                                          cudaMemcpyDeviceToHost, E->xfer));
        }
        CUTC_CUDA_TRY(cudaEventRecord(done[b], E->xfer));
        busy[b] = true;
        return CUTC_OK;
    };
    auto finish_x = [&](int tile) -> int {  // pinned -> pageable caller memory
        if (x_direct)
            return CUTC_OK;
        const int b = tile & 1;
        int64_t i0, nb;
        tile_rows(tile, &i0, &nb);
        CUTC_CUDA_TRY(cudaEventSynchronize(done[b]));
        for (int m = 0; m < R.x_components; m++)
            host_copy(R.X + ((int64_t)m * n1 + i0) * nA2, hpin_x[b] + (int64_t)m * nb * nA2,
                      (size_t)nb * nA2 * 8);
        return CUTC_OK;
    };
    int64_t blk0 = 0;                                  // first r1 row of the int_2e block
    int blk_rows = (int)std::min<int64_t>(kb, n1);     // its rows (whole tiles)
    bool first_blk = true;
    for (int tile = 0; tile < n_tiles; tile++) {
        const int i0 = (int)(tile * n1t);
        const int nb = (int)std::min<int64_t>(n1t, n1 - i0);
        const int ib = (int)(i0 - blk0);  // the tile's first row within the block
        cudaEvent_t *tev = stats ? &E->tile_ev[kTileEv * tile] : nullptr;
        CUTC_TRY(launch_r1_terms(st, i0, nb, nN, d_r1, d_rn, R.a_en, d_t1));
        if (tev)
            CUTC_CUDA_TRY(cudaEventRecord(tev[0], st));
        if (R.precision == CUTC_PLAIN_FP64 || R.pair_fp64) {
            PairArgs P;
            P.i0 = i0; P.n1b = nb; P.n2 = n2; P.nN = nN; P.n_terms = nt;
            P.r1 = d_r1; P.r2 = d_r2; P.t1 = d_t1; P.f2 = d_f2;
            P.coef = d_coef; P.exps = d_exps; P.term_off = d_off;
            P.a_ee = R.a_ee;
            P.G = d_G; P.ldg = n2; P.plane = (int64_t)nb * n2;
            CUTC_TRY(launch_pair_f64(st, P));
            note_launches(2);
            if (R.precision == CUTC_SPLIT_BF16) {
                // the split slicer reads (hi, lo) pairs: convert in place
                CUTC_TRY(launch_f64_to_df(st, d_G, 4 * (int64_t)nb * n2));
                note_launches(1);
            }
        } else {
            PairDfArgs P;
            P.i0 = i0; P.n1b = nb; P.n2 = n2; P.nN = nN; P.rows_per_cta = 0;
            P.r1 = d_r1; P.r2 = d_r2; P.r2d = d_r2d; P.f2 = d_f2; P.f2d = d_f2d; P.t1 = d_t1;
            P.poly = d_poly; P.poly_w = d_poly;
            P.coef = d_coef; P.exps = d_exps; P.term_off = d_off;
            P.a_ee = R.a_ee;
            P.a_ee_hi = (float)R.a_ee;
            P.a_ee_lo = (float)(R.a_ee - (double)P.a_ee_hi);
            P.G = reinterpret_cast<float2 *>(d_G); P.ldg = n2; P.plane = (int64_t)nb * n2;
            // the kernel also leaves the row maxima the G slicer needs
            CUTC_CUDA_TRY(cudaMemsetAsync(sp.BX.rmax, 0, 4 * (size_t)nb * 8, st));
            P.rmax = sp.BX.rmax;
            if (sp.pair_tc) {
                CUTC_TRY(split_pair_tile(E, R, st, sp, P, d_rn, R.a_en));
            } else {
                CUTC_TRY(launch_pair_df(st, P, pexp, psparse, d_rn, R.a_en));
                note_launches(3);
            }
        }
        if (tev)
            CUTC_CUDA_TRY(cudaEventRecord(tev[1], st));
        if (tile == 0 && aos1_deferred) {
            // (from pageable memory the call returns once staged: the GPU is busy meanwhile)
            void *dst = const_cast<double *>(d_aos1);
            if (R.ld1 > n1)  // an r1 window of a larger grid: its 4 nA columns, packed
                CUTC_CUDA_TRY(cudaMemcpy2DAsync(dst, (size_t)n1 * 8, R.aos1, (size_t)R.ld1 * 8,
                                                (size_t)n1 * 8, 4 * (size_t)nA,
                                                cudaMemcpyHostToDevice, E->xfer));
            else
                CUTC_CUDA_TRY(cudaMemcpyAsync(dst, R.aos1, 4 * (size_t)n1 * nA * 8,
                                              cudaMemcpyHostToDevice, E->xfer));
            CUTC_CUDA_TRY(cudaEventRecord(E->ev[6], E->xfer));
        }

        // X rows of the tile into the block:
        //   Xt[(m blk_rows + ib + i) np + p] = sum_g P[p n2 + g] G[m plane + i n2 + g]
        if (R.precision == CUTC_PLAIN_FP64) {
            const double one = 1.0, zero = 0.0;
            if (tev)
                CUTC_CUDA_TRY(cudaEventRecord(tev[2], st));
            CUTC_TRY(fp64_gemm(st, true, (int)np, nb, n2, one, d_P, n2, 0, d_G, n2,
                               (int64_t)nb * n2, zero, d_Xt + (int64_t)ib * np, np,
                               (int64_t)blk_rows * np, 4));
            if (tev)
                CUTC_CUDA_TRY(cudaEventRecord(tev[3], st));
        } else {
            CUTC_TRY(split_x_tile(E, R, st, sp, reinterpret_cast<const float2 *>(d_G), nb, d_Xt,
                                  blk_rows, ib, tev ? tev[2] : nullptr, tev ? tev[3] : nullptr,
                                  !R.pair_fp64));
        }

        // the tile's X rows in the reference layout X[m][i][b][a], before the int_2e share,
        // so that their copy to the host overlaps the int_2e contractions
        if (R.i_only) {
            // X stays packed in the int_2e block and is not returned
        } else if (out_dev) {
            for (int m = 0; m < R.x_components; m++)
                CUTC_TRY(launch_expand_pairs(st, nb, nA, d_Xt + ((int64_t)m * blk_rows + ib) * np,
                                             np, R.X + ((int64_t)m * n1 + i0) * nA2));
        } else {
            const int b = tile & 1;
            if (busy[b])
                CUTC_CUDA_TRY(cudaStreamWaitEvent(st, done[b], 0));
            for (int m = 0; m < R.x_components; m++)
                CUTC_TRY(launch_expand_pairs(st, nb, nA, d_Xt + ((int64_t)m * blk_rows + ib) * np,
                                             np, stage_x[b] + (int64_t)m * nb * nA2));
            CUTC_CUDA_TRY(cudaEventRecord(ready[b], st));
            CUTC_TRY(copy_x(tile));
        }
        if (!R.i_only)
            note_launches(R.x_components);

        // the block's share of int_2e once its last tile is in
        // (src/build_int_2e_ao.cu:60-67 and 97-104, packed):
        //   H += X_3 S0,   N += -1/2 [X_0 X_1 X_2] S   over the block's r1 points
        if (tev)
            CUTC_CUDA_TRY(cudaEventRecord(tev[4], st));
        if (i0 + nb == blk0 + blk_rows && !R.x_only) {
            const int K = blk_rows;
            const double *w1 = d_wr1 + blk0, *a1 = d_aos1 + blk0;
            if (aos1_deferred && first_blk)
                CUTC_CUDA_TRY(cudaStreamWaitEvent(st, E->ev[6], 0));
            if (R.precision == CUTC_PLAIN_FP64) {
                const bool keep =
                    K == n1 && R.mol_tag && E->tag_i == R.mol_tag && E->tag_i_buf == d_S0;
                if (!keep) {
                    CUTC_TRY(launch_sym_products(st, K, nA, w1, a1, ld_a1, d_S0, K));
                    CUTC_TRY(launch_antisym_products(st, K, nA, w1, a1, ld_a1, d_Sl,
                                                     3 * (int64_t)K));
                    note_launches(2);
                }
                E->tag_i = K == n1 ? R.mol_tag : 0;
                E->tag_i_buf = d_S0;
                const double one = 1.0, mhalf = -0.5, beta = first_blk ? 0.0 : 1.0;
                CUTC_TRY(fp64_gemm(st, false, (int)np, (int)np, K, one,
                                   d_Xt + 3 * (int64_t)K * np, np, 0, d_S0, K, 0, beta, d_H, np,
                                   0, 1));
                if (nl > 0)
                    CUTC_TRY(fp64_gemm(st, false, (int)np, (int)nl, 3 * (int64_t)K, mhalf, d_Xt,
                                       np, 0, d_Sl, 3 * (int64_t)K, 0, beta, d_N, np, 0, 1));
            } else {
                CUTC_TRY(split_int2e_tile(E, R, st, sp, w1, a1, ld_a1, K, d_Xt, d_H, d_N,
                                          first_blk));
            }
            first_blk = false;
        }
        if (tev)
            CUTC_CUDA_TRY(cudaEventRecord(tev[5], st));
        // the previous tile's rows, pinned -> pageable, while the device works on this one
        if (!out_dev && !R.i_only && tile > 0)
            CUTC_TRY(finish_x(tile - 1));
        if (i0 + nb == blk0 + blk_rows) {  // next block
            blk0 += blk_rows;
            blk_rows = (int)std::min<int64_t>(kb, n1 - blk0);
        }
    }
    if (!out_dev && n_tiles > 0 && !R.i_only)
        CUTC_TRY(finish_x(n_tiles - 1));
    CUTC_CUDA_TRY(cudaEventRecord(E->ev[5], st));

    // ---- int_2e = A + A^T ------------------------------------------------------
    const bool psqt = R.int2e_layout == CUTC_INT2E_PSQT;
    if (R.x_only) {
        // X alone: nothing to assemble
    } else if (out_dev) {
        CUTC_TRY(launch_assemble_int2e(st, nA, d_H, d_N, 0, (int)nA2, psqt, R.I));
        note_launches(1);
    } else {
        // column slabs: slab s is assembled while slab s - 1 is copied out
        const int n_slabs = (int)((nA2 + slab - 1) / slab);
        bool ibusy[2] = {false, false};
        auto slab_cols = [&](int slab_no, int64_t *c0, int64_t *c1) {
            *c0 = (int64_t)slab_no * slab;
            *c1 = std::min<int64_t>(nA2, *c0 + slab);
        };
        auto copy_i = [&](int slab_no) -> int {
            const int b = slab_no & 1;
            int64_t c0, c1;
            slab_cols(slab_no, &c0, &c1);
            CUTC_CUDA_TRY(cudaStreamWaitEvent(E->xfer, ready[b], 0));
            CUTC_CUDA_TRY(cudaMemcpyAsync(i_direct ? R.I + c0 * nA2 : hpin_i[b], stage_i[b],
                                          (size_t)(c1 - c0) * nA2 * 8, cudaMemcpyDeviceToHost,
                                          E->xfer));
            CUTC_CUDA_TRY(cudaEventRecord(done[b], E->xfer));
            ibusy[b] = true;
            return CUTC_OK;
        };
        auto finish_i = [&](int slab_no) -> int {
            if (i_direct)
                return CUTC_OK;
            const int b = slab_no & 1;
            int64_t c0, c1;
            slab_cols(slab_no, &c0, &c1);
            CUTC_CUDA_TRY(cudaEventSynchronize(done[b]));
            host_copy(R.I + c0 * nA2, hpin_i[b], (size_t)(c1 - c0) * nA2 * 8);
            return CUTC_OK;
        };
        // the X copies still pending on the staging events must be waited for
        // before those events are recorded again
        for (int b = 0; b < 2; b++)
            if (busy[b])
                CUTC_CUDA_TRY(cudaStreamWaitEvent(st, done[b], 0));
        for (int sl = 0; sl < n_slabs; sl++) {
            const int b = sl & 1;
            int64_t c0, c1;
            slab_cols(sl, &c0, &c1);
            if (ibusy[b])
                CUTC_CUDA_TRY(cudaStreamWaitEvent(st, done[b], 0));
            CUTC_TRY(launch_assemble_int2e(st, nA, d_H, d_N, (int)c0, (int)c1, psqt, stage_i[b]));
            note_launches(1);
            CUTC_CUDA_TRY(cudaEventRecord(ready[b], st));
            CUTC_TRY(copy_i(sl));
            if (sl > 0)
                CUTC_TRY(finish_i(sl - 1));
        }
        CUTC_TRY(finish_i(n_slabs - 1));
    }
    CUTC_CUDA_TRY(cudaEventRecord(E->ev[7], st));
    CUTC_CUDA_TRY(cudaEventRecord(E->ev[11], E->xfer));
    CUTC_CUDA_TRY(cudaStreamWaitEvent(st, E->ev[11], 0));
    CUTC_CUDA_TRY(cudaEventRecord(E->ev[8], st));
    CUTC_CUDA_TRY(cudaEventSynchronize(E->ev[8]));
    CUTC_CUDA_TRY(cudaGetLastError());
    if (R.precision == CUTC_SPLIT_BF16)
        CUTC_TRY(split_check(st, sp));

    if (stats) {
        double ms_pair = 0.0, ms_gemm = 0.0, ms_i = 0.0, ms_tiles = 0.0;
        for (int t = 0; t < n_tiles; t++) {
            const cudaEvent_t *e = &E->tile_ev[kTileEv * t];
            ms_pair += ev_ms(e[0], e[1]);
            ms_gemm += ev_ms(e[2], e[3]);
            ms_i += ev_ms(e[4], e[5]);
            ms_tiles += ev_ms(e[0], e[5]);
        }
        // a tile's X contraction is one FP64 launch, or the split form's K launches
        int x_launches = 1;
        if (R.precision == CUTC_SPLIT_BF16) {
            const int64_t nkb = ((int64_t)R.n2 + 31) / 32;
            const int64_t per = split_k_blocks_per_launch(nkb * 32, n_pairs(R.nA), R.k_split);
            x_launches = (int)((nkb + per - 1) / per);
        }
        stats->ms_x_gemm = ms_gemm;
        stats->n_x_gemm = n_tiles * x_launches;
        stats->ms_h2d = ev_ms(E->ev[0], E->ev[1]);
        stats->ms_pair = ms_pair;
        stats->ms_x = ev_ms(E->ev[1], E->ev[2]) + ms_tiles - ms_pair - ms_i;
        stats->ms_int2e = ms_i + ev_ms(E->ev[5], E->ev[7]);
        stats->ms_d2h = ev_ms(E->ev[7], E->ev[8]);
        stats->ms_total = ev_ms(E->ev[0], E->ev[8]);
        stats->n_r1_tiles = n_tiles;
        stats->gpu_launches = (int)(launches_so_far() - launches0);
    }
    if (default_budget) {  // completed: the buffers of this shape hold this plan
        memo.key = key;
        memo.path = path;
        memo.budget = budget;
        memo.n1t = n1t;
        memo.kb = kb;
        E->ws.remember(memo);
    }
    return CUTC_OK;
}

// The pair terms alone, on device arrays: rows [i0, i0 + n1b) of r1 against the
// r2 points [j0, j0 + n2b) of r2, into G[c * plane + i * ldg + j] (c = 0..3).
int run_pair_only(Engine *E, cudaStream_t st, int i0, int n1b, int n1, int j0, int n2b,
                  int64_t ldg, int64_t plane, int nN, int nB, const double *r1, const double *r2,
                  const double *rn, const double *c_bh, const int *m_bh, const int *n_bh,
                  const int *o_bh, double a_en, double a_ee, double *G)
{
    if (n1b <= 0 || n2b <= 0 || nN <= 0 || nB < 0 || i0 < 0 || j0 < 0 || i0 + n1b > n1 ||
        nN > kMaxNuc || ldg < n2b || plane < (n1b - 1) * ldg + n2b || !r1 || !r2 || !rn || !G ||
        !(a_en > 0) || !(a_ee > 0)) {
        cutc_set_error(CUTC_ERR_INVALID, "invalid pair-kernel arguments");
        return CUTC_ERR_INVALID;
    }
    // parameters come from the device: bring them to the host to build the term table
    std::vector<double> c((size_t)nN * nB);
    std::vector<int> m((size_t)nN * nB), n((size_t)nN * nB), o((size_t)nN * nB);
    if (nB > 0) {
        CUTC_CUDA_TRY(cudaMemcpyAsync(c.data(), c_bh, c.size() * 8, cudaMemcpyDeviceToHost, st));
        CUTC_CUDA_TRY(cudaMemcpyAsync(m.data(), m_bh, m.size() * 4, cudaMemcpyDeviceToHost, st));
        CUTC_CUDA_TRY(cudaMemcpyAsync(n.data(), n_bh, n.size() * 4, cudaMemcpyDeviceToHost, st));
        CUTC_CUDA_TRY(cudaMemcpyAsync(o.data(), o_bh, o.size() * 4, cudaMemcpyDeviceToHost, st));
        CUTC_CUDA_TRY(cudaStreamSynchronize(st));
    }
    Request R{};
    R.nN = nN; R.nB = nB; R.c_bh = c.data(); R.m_bh = m.data(); R.n_bh = n.data(); R.o_bh = o.data();
    std::vector<double> coef;
    std::vector<int> exps, off;
    CUTC_TRY(build_terms(R, coef, exps, off));
    Workspace &W = E->ws;
    void *p;
    CUTC_TRY(W.get(S_COEF, std::max<size_t>(1, coef.size()) * 8, &p));
    double *d_coef = (double *)p;
    CUTC_TRY(W.get(S_EXPS, std::max<size_t>(1, exps.size()) * 4, &p));
    int *d_exps = (int *)p;
    CUTC_TRY(W.get(S_OFF, off.size() * 4, &p));
    int *d_off = (int *)p;
    if (!exps.empty()) {
        CUTC_CUDA_TRY(cudaMemcpyAsync(d_coef, coef.data(), coef.size() * 8, cudaMemcpyHostToDevice, st));
        CUTC_CUDA_TRY(cudaMemcpyAsync(d_exps, exps.data(), exps.size() * 4, cudaMemcpyHostToDevice, st));
    }
    CUTC_CUDA_TRY(cudaMemcpyAsync(d_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice, st));
    CUTC_TRY(W.get(S_T1, (size_t)n1b * nN * sizeof(NucTerm), &p));
    NucTerm *d_t1 = (NucTerm *)p;
    CUTC_TRY(W.get(S_F2, (size_t)nN * n2b * 8, &p));
    double *d_f2 = (double *)p;
    const double *r2w = r2 + 3 * (int64_t)j0;  // the r2 window
    CUTC_TRY(launch_r1_terms(st, i0, n1b, nN, r1, rn, a_en, d_t1));
    CUTC_TRY(launch_r2_terms(st, n2b, nN, r2w, rn, a_en, d_f2));
    PairArgs P;
    P.i0 = i0; P.n1b = n1b; P.n2 = n2b; P.nN = nN; P.n_terms = (int)exps.size();
    P.r1 = r1; P.r2 = r2w; P.t1 = d_t1; P.f2 = d_f2;
    P.coef = d_coef; P.exps = d_exps; P.term_off = d_off; P.a_ee = a_ee;
    P.G = G; P.ldg = ldg; P.plane = plane;
    CUTC_TRY(launch_pair_f64(st, P));
    note_launches(3);
    CUTC_CUDA_TRY(cudaStreamSynchronize(st));
    return CUTC_OK;
}

}  // namespace cutc

// ---------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------
using namespace cutc;

extern "C" void cutc_default_options(cutc_options *opt)
{
    memset(opt, 0, sizeof(*opt));
    opt->precision = CUTC_PLAIN_FP64;
    opt->n_slices = kDefaultSlices;
    opt->a_en = 1.0;
    opt->a_ee = 1.0;
    opt->x_components = 3;
}

extern "C" int cutc_int_ex(const cutc_options *opt, int n_grid1, int n_grid2, int n_ao, int n_nuc,
                           int size_bh, const double *r1, const double *wr1, const double *r2,
                           const double *wr2, const double *rn, const double *aos_data1,
                           const double *aos_data2, const double *c_bh, const int *m_bh,
                           const int *n_bh, const int *o_bh, double *int2_grad1_u12_ao,
                           double *int_2e_ao, cutc_stats *stats)
{
    cutc_options defaults;
    if (!opt) {
        cutc_default_options(&defaults);
        opt = &defaults;
    }
    Engine *E = nullptr;
    CUTC_TRY(get_engine(&E));
    Request R{};
    R.precision = opt->precision;
    R.n_slices = opt->n_slices;
    R.a_en = opt->a_en;
    R.a_ee = opt->a_ee;
    R.x_components = opt->x_components;
    R.device_pointers = opt->device_pointers;
    R.max_work_bytes = opt->max_work_bytes;
    R.stream = (cudaStream_t)opt->stream;
    R.pair_fp64 = opt->pair_fp64;
    R.k_split = opt->k_split;
    R.int2e_layout = opt->int2e_layout;
    R.basis = opt->basis;
    R.n1 = n_grid1; R.n2 = n_grid2; R.nA = n_ao; R.nN = n_nuc; R.nB = size_bh;
    R.r1 = r1; R.wr1 = wr1; R.r2 = r2; R.wr2 = wr2; R.rn = rn;
    R.aos1 = aos_data1; R.aos2 = aos_data2;
    R.c_bh = c_bh; R.m_bh = m_bh; R.n_bh = n_bh; R.o_bh = o_bh;
    R.X = int2_grad1_u12_ao; R.I = int_2e_ao;
    R.x_only = int_2e_ao == nullptr;
    R.i_only = int2_grad1_u12_ao == nullptr;
    if (opt->r1_begin != 0 || opt->r1_end != 0) {
        // an r1 shard: the window's points of the full arrays
        if (opt->r1_begin < 0 || opt->r1_end <= opt->r1_begin || opt->r1_end > n_grid1) {
            cutc_set_error(CUTC_ERR_INVALID, "r1 window [%d, %d) outside [0, n_grid1=%d)",
                           opt->r1_begin, opt->r1_end, n_grid1);
            return CUTC_ERR_INVALID;
        }
        const int b = opt->r1_begin;
        R.n1 = opt->r1_end - b;
        if (R.r1)
            R.r1 += 3 * (int64_t)b;
        if (R.wr1)
            R.wr1 += b;
        if (R.aos1) {
            R.aos1 += b;
            R.ld1 = n_grid1;
        }
    }
    const char *tr = getenv("CUTC_TILE_ROWS");
    R.tile_rows = tr ? atoi(tr) : 0;
    const char *ir = getenv("CUTC_INT2E_ROWS");
    R.int2e_rows = ir ? atoi(ir) : 0;
    if (stats)
        memset(stats, 0, sizeof(*stats));
    std::lock_guard<std::mutex> lk(E->mu);
    int s = run_build(E, R, stats);
    if (s != CUTC_OK)
        cudaStreamSynchronize(R.stream ? R.stream : E->stream);
    return s;
}

extern "C" int cutc_int_scan(const cutc_options *opt, int n_sets, int n_grid1, int n_grid2,
                             int n_ao, int n_nuc, int size_bh, const double *r1, const double *wr1,
                             const double *r2, const double *wr2, const double *rn,
                             const double *aos_data1, const double *aos_data2, const double *c_bh,
                             const int *m_bh, const int *n_bh, const int *o_bh,
                             const double *a_en, const double *a_ee, double *int2_grad1_u12_ao,
                             double *int_2e_ao, cutc_stats *stats)
{
    cutc_options defaults;
    if (!opt) {
        cutc_default_options(&defaults);
        opt = &defaults;
    }
    if (n_sets < 1 || n_grid1 <= 0 || n_grid2 <= 0 || n_ao <= 0 || n_nuc <= 0 || size_bh < 0 ||
        !int2_grad1_u12_ao || !int_2e_ao || opt->r1_begin != 0 || opt->r1_end != 0) {
        cutc_set_error(CUTC_ERR_INVALID, "invalid scan arguments (an r1 window is not taken)");
        return CUTC_ERR_INVALID;
    }
    static std::atomic<unsigned long long> next_tag{1};
    const uint64_t tag = next_tag.fetch_add(1);
    Engine *E = nullptr;
    CUTC_TRY(get_engine(&E));
    std::lock_guard<std::mutex> lk(E->mu);
    Request base{};
    base.precision = opt->precision;
    base.n_slices = opt->n_slices;
    base.x_components = opt->x_components;
    base.device_pointers = opt->device_pointers;
    base.max_work_bytes = opt->max_work_bytes;
    base.stream = (cudaStream_t)opt->stream;
    base.pair_fp64 = opt->pair_fp64;
    base.k_split = opt->k_split;
    base.int2e_layout = opt->int2e_layout;
    base.basis = opt->basis;
    base.n1 = n_grid1; base.n2 = n_grid2; base.nA = n_ao; base.nN = n_nuc; base.nB = size_bh;
    base.r1 = r1; base.wr1 = wr1; base.r2 = r2; base.wr2 = wr2; base.rn = rn;
    base.aos1 = aos_data1; base.aos2 = aos_data2;
    base.mol_tag = tag;
    cudaStream_t st = base.stream ? base.stream : E->stream;
    if (!opt->device_pointers) {
        // the molecule arrays go to the device once for all parameter sets
        if (!r1 || !wr1 || !r2 || !wr2 || !rn || ((!aos_data1 || !aos_data2) && !opt->basis)) {
            cutc_set_error(CUTC_ERR_INVALID, "NULL array argument");
            return CUTC_ERR_INVALID;
        }
        struct { int slot; const double *src; size_t n; const double **dst; } up[] = {
            {150, r1, 3 * (size_t)n_grid1, &base.r1}, {151, wr1, (size_t)n_grid1, &base.wr1},
            {152, r2, 3 * (size_t)n_grid2, &base.r2}, {153, wr2, (size_t)n_grid2, &base.wr2},
            {154, rn, 3 * (size_t)n_nuc, &base.rn},
            {155, aos_data1, 4 * (size_t)n_grid1 * n_ao, &base.aos1},
            {156, aos_data2, (size_t)n_grid2 * n_ao, &base.aos2}};
        for (auto &u : up) {
            if (!u.src)
                continue;  // evaluated from the basis below
            void *p = nullptr;
            CUTC_TRY(E->ws.get(u.slot, u.n * sizeof(double), &p));
            CUTC_CUDA_TRY(cudaMemcpyAsync(p, u.src, u.n * sizeof(double), cudaMemcpyHostToDevice, st));
            *u.dst = (const double *)p;
        }
        base.in_device = 1;
    }
    if (!base.aos1 || !base.aos2) {
        // every set shares the molecule: evaluate its AOs once
        if (!opt->basis) {
            cutc_set_error(CUTC_ERR_INVALID, "NULL AO array and no basis to evaluate it from");
            return CUTC_ERR_INVALID;
        }
        CUTC_TRY(validate_basis(opt->basis, n_ao));
        BasisDev B;
        CUTC_TRY(upload_basis(E->ws, 157, st, opt->basis, &B));
        void *p = nullptr;
        if (!base.aos1) {
            CUTC_TRY(E->ws.get(155, 4 * (size_t)n_grid1 * n_ao * sizeof(double), &p));
            CUTC_TRY(launch_eval_aos(st, B, n_grid1, base.r1, 4, (double *)p, n_grid1));
            base.aos1 = (const double *)p;
        }
        if (!base.aos2) {
            CUTC_TRY(E->ws.get(156, (size_t)n_grid2 * n_ao * sizeof(double), &p));
            CUTC_TRY(launch_eval_aos(st, B, n_grid2, base.r2, 1, (double *)p, n_grid2));
            base.aos2 = (const double *)p;
        }
        base.in_device = 1;
    }
    if (stats)
        memset(stats, 0, sizeof(*stats));
    const size_t nt = (size_t)size_bh * n_nuc;
    const size_t xs = (size_t)opt->x_components * n_grid1 * n_ao * n_ao;
    const size_t is = (size_t)n_ao * n_ao * n_ao * n_ao;
    for (int s = 0; s < n_sets; s++) {
        Request R = base;
        R.c_bh = c_bh + s * nt;
        R.m_bh = m_bh + s * nt;
        R.n_bh = n_bh + s * nt;
        R.o_bh = o_bh + s * nt;
        R.a_en = a_en ? a_en[s] : opt->a_en;
        R.a_ee = a_ee ? a_ee[s] : opt->a_ee;
        R.X = int2_grad1_u12_ao + s * xs;
        R.I = int_2e_ao + s * is;
        cutc_stats one;
        int rc = run_build(E, R, stats ? &one : nullptr);
        if (rc != CUTC_OK) {
            cudaStreamSynchronize(st);
            E->tag_x = E->tag_i = 0;
            return rc;
        }
        if (stats) {
            stats->ms_total += one.ms_total;
            stats->ms_h2d += one.ms_h2d;
            stats->ms_pair += one.ms_pair;
            stats->ms_x += one.ms_x;
            stats->ms_int2e += one.ms_int2e;
            stats->ms_d2h += one.ms_d2h;
            stats->n_r1_tiles += one.n_r1_tiles;
            stats->gpu_launches += one.gpu_launches;
            stats->ms_x_gemm += one.ms_x_gemm;
            stats->n_x_gemm += one.n_x_gemm;
        }
    }
    E->tag_x = E->tag_i = 0;
    return CUTC_OK;
}

extern "C" int cutc_check_wait_limit(void)
{
    Engine *E = nullptr;
    CUTC_TRY(get_engine(&E));
    std::lock_guard<std::mutex> lk(E->mu);
    return split_wait_limit_check(E);
}

extern "C" int cutc_jast_bh_dev(int i0, int n1b, int n_grid1, int n_grid2, int n_nuc, int size_bh,
                                const double *r1, const double *r2, const double *rn,
                                const double *c_bh, const int *m_bh, const int *n_bh,
                                const int *o_bh, double a_en, double a_ee, double *grad1u)
{
    Engine *E = nullptr;
    CUTC_TRY(get_engine(&E));
    std::lock_guard<std::mutex> lk(E->mu);
    return run_pair_only(E, E->stream, i0, n1b, n_grid1, 0, n_grid2, n_grid2,
                         (int64_t)n1b * n_grid2, n_nuc, size_bh, r1, r2, rn, c_bh, m_bh, n_bh,
                         o_bh, a_en, a_ee, grad1u);
}

extern "C" int cutc_split_gemm_dev(int n_slices, int M, int N, long long K, const double *A,
                                   const double *B, double *C, long long ldc)
{
    if (M <= 0 || N <= 0 || K <= 0 || !A || !B || !C || ldc < M || n_slices < 3 ||
        n_slices > kMaxSlices) {
        cutc_set_error(CUTC_ERR_INVALID, "invalid split GEMM arguments");
        return CUTC_ERR_INVALID;
    }
    Engine *E = nullptr;
    CUTC_TRY(get_engine(&E));
    std::lock_guard<std::mutex> lk(E->mu);
    return split_gemm_dense(E, E->stream, n_slices, M, N, K, A, B, C, ldc);
}

extern "C" int cutc_fp64_gemm_dev(int a_kmajor, int M, int N, long long K, double alpha,
                                  const double *A, long long lda, long long stride_a,
                                  const double *B, long long ldb, long long stride_b, double beta,
                                  double *C, long long ldc, long long stride_c, int batch)
{
    Engine *E = nullptr;
    CUTC_TRY(get_engine(&E));
    std::lock_guard<std::mutex> lk(E->mu);
    CUTC_TRY(fp64_gemm(E->stream, a_kmajor != 0, M, N, K, alpha, A, lda, stride_a, B, ldb,
                       stride_b, beta, C, ldc, stride_c, batch));
    CUTC_CUDA_TRY(cudaStreamSynchronize(E->stream));
    return CUTC_OK;
}

extern "C" int cutc_validate_launch_dims(int gx, int gy, int gz, int bx, int by, int bz)
{
    Engine *E = nullptr;
    CUTC_TRY(get_engine(&E));
    // The reference compares unsigned dim3 products with the device limits
    // (src/cutc_int.c:79-86); the same unsigned arithmetic is kept here.
    const unsigned vol = (unsigned)bx * (unsigned)by * (unsigned)bz;
    if (vol > (unsigned)E->max_threads_per_block) {
        cutc_set_error(CUTC_ERR_LAUNCH_DIMS, "Too many threads per block");
        return CUTC_ERR_LAUNCH_DIMS;
    }
    if ((unsigned)gx > (unsigned)E->max_grid[0] || (unsigned)gy > (unsigned)E->max_grid[1] ||
        (unsigned)gz > (unsigned)E->max_grid[2]) {
        cutc_set_error(CUTC_ERR_LAUNCH_DIMS, "Grid dimensions exceed device capabilities");
        return CUTC_ERR_LAUNCH_DIMS;
    }
    return CUTC_OK;
}

extern "C" void cutc_release(void)
{
    Engine *E = nullptr;
    if (get_engine(&E) != CUTC_OK)
        return;
    std::lock_guard<std::mutex> lk(E->mu);
    cudaStreamSynchronize(E->stream);
    cudaStreamSynchronize(E->xfer);
    E->ws.release();
    E->pinned.release();
    E->tag_x = E->tag_i = 0;  // the operands they name are gone
}

extern "C" int cutc_eval_aos(const cutc_basis *basis, int n_points, const double *r,
                             int components, double *aos, int device_pointers, void *stream)
{
    using namespace cutc;
    if (n_points < 0 || !r || !aos || (components != 1 && components != 4)) {
        cutc_set_error(CUTC_ERR_INVALID, "invalid AO evaluation arguments");
        return CUTC_ERR_INVALID;
    }
    CUTC_TRY(validate_basis(basis, basis ? basis->n_ao : 0));
    Engine *E = nullptr;
    CUTC_TRY(get_engine(&E));
    std::lock_guard<std::mutex> lk(E->mu);
    cudaStream_t st = stream ? (cudaStream_t)stream : E->stream;
    BasisDev B;
    CUTC_TRY(upload_basis(E->ws, 160, st, basis, &B));
    if (n_points == 0)
        return CUTC_OK;
    const size_t out_bytes = (size_t)components * basis->n_ao * n_points * sizeof(double);
    if (device_pointers)
        return launch_eval_aos(st, B, n_points, r, components, aos, n_points);
    void *pr = nullptr, *po = nullptr;
    CUTC_TRY(E->ws.get(161, 3 * (size_t)n_points * sizeof(double), &pr));
    CUTC_TRY(E->ws.get(162, out_bytes, &po));
    CUTC_CUDA_TRY(cudaMemcpyAsync(pr, r, 3 * (size_t)n_points * sizeof(double),
                                  cudaMemcpyHostToDevice, st));
    CUTC_TRY(launch_eval_aos(st, B, n_points, (const double *)pr, components, (double *)po,
                             n_points));
    CUTC_CUDA_TRY(cudaMemcpyAsync(aos, po, out_bytes, cudaMemcpyDeviceToHost, st));
    CUTC_CUDA_TRY(cudaStreamSynchronize(st));
    return CUTC_OK;
}

extern "C" int cutc_plan(const cutc_options *opt, int n_grid1, int n_grid2, int n_ao, int n_nuc,
                         cutc_plan_info *plan)
{
    using namespace cutc;
    cutc_options defaults;
    if (!opt) {
        cutc_default_options(&defaults);
        opt = &defaults;
    }
    if (!plan || n_grid1 <= 0 || n_grid2 <= 0 || n_ao <= 0 || n_nuc <= 0 ||
        (opt->precision == CUTC_SPLIT_BF16 && (opt->n_slices < 3 || opt->n_slices > kMaxSlices)) ||
        (opt->x_components != 3 && opt->x_components != 4)) {
        cutc_set_error(CUTC_ERR_INVALID, "invalid plan arguments");
        return CUTC_ERR_INVALID;
    }
    Request R{};
    R.precision = opt->precision;
    R.n_slices = opt->n_slices;
    R.x_components = opt->x_components;
    R.device_pointers = opt->device_pointers;
    R.n1 = n_grid1; R.n2 = n_grid2; R.nA = n_ao; R.nN = n_nuc;
    if (const char *tr = getenv("CUTC_TILE_ROWS"))
        R.tile_rows = atoi(tr);
    if (const char *ir = getenv("CUTC_INT2E_ROWS"))
        R.int2e_rows = atoi(ir);
    size_t budget = opt->max_work_bytes;
    int64_t n1t, kb;
    PlanMemo memo;
    if (budget == 0 && engine_recall(plan_key(R), &memo)) {
        budget = memo.budget;  // as a build of this shape on the device's engine would
        n1t = memo.n1t;
        kb = memo.kb;
    } else {
        if (budget == 0) {
            size_t free_b = 0, total_b = 0;
            cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
            if (e != cudaSuccess) {
                cudaGetLastError();
                cutc_set_error(CUTC_ERR_NO_DEVICE, "no device to size the default budget: %s",
                               cudaGetErrorString(e));
                return CUTC_ERR_NO_DEVICE;
            }
            budget = std::min<size_t>((size_t)24 << 30, free_b / 4);
            const size_t fixed = fixed_bytes(R);
            if (free_b > fixed)
                budget = std::min<size_t>(budget, (size_t)((double)(free_b - fixed) * 0.4));
        }
        plan_rows(R, budget, &n1t, &kb);
    }
    plan->tile_rows = (int)n1t;
    plan->block_rows = (int)kb;
    plan->n_tiles = (int)((n_grid1 + n1t - 1) / n1t);
    plan->n_blocks = (int)((n_grid1 + kb - 1) / kb);
    plan->slab_cols = int2e_slab_cols(n_ao);
    plan->budget_bytes = budget;
    plan->fixed_bytes = fixed_bytes(R);
    plan->tile_row_bytes = r1_row_bytes(R);
    plan->block_row_bytes = int2e_row_bytes(R);
    plan->footprint_bytes = build_footprint(R, budget);
    if (R.precision == CUTC_SPLIT_BF16) {
        const int64_t nkb = ((int64_t)n_grid2 + 31) / 32;
        const int64_t per = split_k_blocks_per_launch(nkb * 32, n_pairs(n_ao), opt->k_split);
        plan->x_launches_per_tile = (int)((nkb + per - 1) / per);
    } else {
        plan->x_launches_per_tile = 1;  // one FP64 GEMM launch over the four components
    }
    return CUTC_OK;
}

extern "C" int cutc_pin_host(void *ptr, size_t bytes)
{
    if (!ptr || bytes == 0) {
        cutc_set_error(CUTC_ERR_INVALID, "nothing to pin");
        return CUTC_ERR_INVALID;
    }
    CUTC_CUDA_TRY(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
    return CUTC_OK;
}

extern "C" int cutc_unpin_host(void *ptr)
{
    if (!ptr) {
        cutc_set_error(CUTC_ERR_INVALID, "nothing to unpin");
        return CUTC_ERR_INVALID;
    }
    CUTC_CUDA_TRY(cudaHostUnregister(ptr));
    return CUTC_OK;
}
