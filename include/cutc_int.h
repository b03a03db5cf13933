/*
 * cutc_int.h -- C-ABI of the GB300 transcorrelated-integral engine
 * (libcutcint.so, built for sm_103a).
 *
 * Drop-in surface: `cutc_int` keeps the argument list, array layouts and
 * return codes of CuTC's entry point (src/cutc_int.c:15-20, declared for
 * Fortran in src/cutc_module.f90:10-39).  Everything else in this header is an
 * extension with plain pointers and sizes only.
 *
 * Array layouts (Fortran column-major, FP64 unless noted):
 *   r1(3, n_grid1)   wr1(n_grid1)   r2(3, n_grid2)   wr2(n_grid2)   rn(3, n_nuc)
 *   aos_data1(n_grid1, n_ao, 4)     aos_data2(n_grid2, n_ao, 4)   [value, d/dx, d/dy, d/dz]
 *   c_bh(size_bh, n_nuc)   m_bh, n_bh, o_bh(size_bh, n_nuc) int32, exponents in [0, 6]
 * Outputs:
 *   int2_grad1_u12_ao(n_ao, n_ao, n_grid1, 3)   X_{mu nu}(r1) = sum_r2 w2 chi_mu chi_nu grad1 u
 *   int_2e_ao(n_ao, n_ao, n_ao, n_ao)           two-electron TC integrals (A + A^T)
 */
#ifndef CUTC_GB300_CUTC_INT_H
#define CUTC_GB300_CUTC_INT_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define CUTC_OK 0
#define CUTC_ERR_LAUNCH_DIMS (-1) /* same code and condition as src/cutc_int.c:79-86 */
#define CUTC_ERR_INVALID (-2)     /* bad size, NULL pointer, exponent outside [0, 6] */
#define CUTC_ERR_NO_MEMORY (-3)   /* device memory exhausted even after tiling */
#define CUTC_ERR_CUDA (-4)        /* CUDA failure (message in cutc_last_error) */
#define CUTC_ERR_NO_DEVICE (-5)   /* no usable sm_103 GPU */
#define CUTC_ERR_TIMEOUT (-6)     /* a bounded device-side wait gave up */

/* ---- precision forms --------------------------------------------------- */
#define CUTC_PLAIN_FP64 0 /* FP64 contractions: the drop-in form */
#define CUTC_SPLIT_BF16 1 /* FP64 operands split into BF16 slices on tcgen05, exact FP32 sums, FP64 result */

/*
 * Drop-in replacement for CuTC's cutc_int (src/cutc_int.c:15-20).
 * All pointers are host pointers (pageable is fine).  The six launch integers
 * are validated exactly as the reference does (block volume against the
 * device's maxThreadsPerBlock, grid against maxGridSize; -1 on failure) and
 * are otherwise ignored: the engine picks its own launch geometry.
 * Only the first three components of X are written, as in the reference
 * (src/cutc_int.c:105,210).  Computes in the plain FP64 form.
 * Returns CUTC_OK or a negative status; never calls exit().
 */
int cutc_int(int nxBlocks, int nyBlocks, int nzBlocks,
             int blockxSize, int blockySize, int blockzSize,
             int n_grid1, int n_grid2, int n_ao, int n_nuc, int size_bh,
             double *r1, double *wr1, double *r2, double *wr2, double *rn,
             double *aos_data1, double *aos_data2,
             double *c_bh, int *m_bh, int *n_bh, int *o_bh,
             double *int2_grad1_u12_ao, double *int_2e_ao);

/* ---- extended API (no reference counterpart) --------------------------- */

/* A Cartesian Gaussian basis, one entry per atomic orbital (host memory):
 *   chi_a(r) = x^lx y^ly z^lz sum_k c_k exp(-alpha_k |r - C_a|^2),  (x,y,z) = r - C_a,
 * with k = prim_offset[a] .. prim_offset[a+1]-1, normalisation folded into
 * c_k, powers 0..8, 1..64 primitives per function. */
typedef struct cutc_basis {
    int n_ao;
    const double *center;       /* (3, n_ao): C_a */
    const int *power;           /* (3, n_ao): lx, ly, lz */
    const int *prim_offset;     /* (n_ao + 1), prim_offset[0] = 0 */
    const double *prim_exp;     /* alpha_k */
    const double *prim_coef;    /* c_k */
} cutc_basis;

typedef struct cutc_options {
    int precision;          /* CUTC_PLAIN_FP64 or CUTC_SPLIT_BF16 */
    int n_slices;           /* split form: BF16 slices per operand, 3..7 (default 5) */
    double a_en;            /* e-n Jastrow scale: f = a r / (1 + a r); 1.0 = reference */
    double a_ee;            /* e-e Jastrow scale; 1.0 = reference */
    int x_components;       /* X components copied out: 3 (reference) or 4 */
    int device_pointers;    /* 1: every array argument is a device pointer */
    size_t max_work_bytes;  /* device budget for the r1 tiles; 0 = automatic */
    void *stream;           /* cudaStream_t to run on; NULL = the engine's stream */
    int pair_fp64;          /* split form: 1 = pair terms in FP64 instead of double-float */
    int k_split;            /* split form: max K per tensor-core launch; the partial results
                               are summed in FP64 (0 = automatic: one launch up to K = 65536,
                               equal launches of at most 49152 beyond) */
    int int2e_layout;       /* CUTC_INT2E_PQST (reference order) or CUTC_INT2E_PSQT: int_2e with
                               its 2nd and 3rd indices swapped, as trans_pqst_psqt_inplace
                               leaves it (the order cutc_no uses), written directly */
    const cutc_basis *basis;    /* with aos_data1 and/or aos_data2 NULL: those AO arrays are
                                   evaluated on the device from this basis (NULL: not used) */
    int r1_begin, r1_end;   /* cutc_int_ex only: an r1 shard.  With r1_end > r1_begin the build
                               covers r1 points [r1_begin, r1_end) of the full arrays r1, wr1 and
                               aos_data1 (still laid out for all n_grid1 points); X is written for
                               those points only, as X(n_ao, n_ao, r1_end - r1_begin, comps),
                               and int_2e receives that shard's share A_s + A_s^T.  int_2e is
                               linear in the r1 points, so the shares of shards that partition
                               [0, n_grid1) sum to the whole build's int_2e (the r1 sharding of
                               a build over several GPUs; the caller sums the shares, e.g. with
                               one all-reduce).  0, 0 = the whole grid */
} cutc_options;

#define CUTC_INT2E_PQST 0
#define CUTC_INT2E_PSQT 1

typedef struct cutc_stats {
    double ms_total;        /* wall time of the call */
    double ms_h2d;          /* host -> device copies */
    double ms_pair;         /* pair terms (grad1 u) */
    double ms_x;            /* X contraction(s) incl. slicing */
    double ms_int2e;        /* int_2e contraction(s) + assembly */
    double ms_d2h;          /* device -> host copies */
    int n_r1_tiles;         /* r1 tiles the X build was split into */
    int gpu_launches;       /* kernels of this library launched by the call */
    double ms_x_gemm;       /* device time of the X-build contraction launches alone */
    int n_x_gemm;           /* number of those launches: one per r1 tile (plain form),
                               the K launches of each r1 tile (split form) */
} cutc_stats;

/* Fills the defaults: plain FP64, 5 slices, a_en = a_ee = 1, 3 X components. */
void cutc_default_options(cutc_options *opt);

/*
 * cutc_int with options.  With opt->device_pointers = 1 all array arguments
 * (inputs and outputs) are device pointers on the current device and no
 * host<->device copies are made.  stats may be NULL.  int_2e_ao may be NULL:
 * then only X is built (opt->x_components of them), and wr1 and aos_data1 are
 * not read and may be NULL too.  int2_grad1_u12_ao may be NULL instead: then
 * only int_2e is returned (X is formed on the device in the packed layout the
 * contractions use and is not expanded or copied out), for builds whose X would
 * not fit beside the working set or is not needed.
 */
int cutc_int_ex(const cutc_options *opt,
                int n_grid1, int n_grid2, int n_ao, int n_nuc, int size_bh,
                const double *r1, const double *wr1, const double *r2, const double *wr2,
                const double *rn, const double *aos_data1, const double *aos_data2,
                const double *c_bh, const int *m_bh, const int *n_bh, const int *o_bh,
                double *int2_grad1_u12_ao, double *int_2e_ao, cutc_stats *stats);

/*
 * A Jastrow-parameter scan: the build of cutc_int_ex for n_sets parameter sets
 * on one molecule.  The molecule arrays are copied to the device once and the
 * Jastrow-independent operands (the AO pair products on both grids, or their
 * BF16 slices) are built once and shared by all sets; only the pair terms and
 * the contractions run per set.  Set s uses c/m/n/o_bh + s * size_bh * n_nuc,
 * a_en[s] and a_ee[s] (NULL: opt->a_en / opt->a_ee) and writes its outputs at
 * int2_grad1_u12_ao + s * x_components * n_grid1 * n_ao^2 and
 * int_2e_ao + s * n_ao^4.  Each set's result equals the cutc_int_ex result
 * with the same options.  stats (optional) sums the per-set statistics.
 * No reference counterpart.
 */
int cutc_int_scan(const cutc_options *opt, int n_sets,
                  int n_grid1, int n_grid2, int n_ao, int n_nuc, int size_bh,
                  const double *r1, const double *wr1, const double *r2, const double *wr2,
                  const double *rn, const double *aos_data1, const double *aos_data2,
                  const double *c_bh, const int *m_bh, const int *n_bh, const int *o_bh,
                  const double *a_en, const double *a_ee,
                  double *int2_grad1_u12_ao, double *int_2e_ao, cutc_stats *stats);

/*
 * Pair terms alone, on device pointers: for r1 rows [i0, i0 + n1b) and all
 * r2 points, writes grad1u[c * n1b * n2 + i * n2 + j] for c = 0..2 (gradient)
 * and c = 3 (-1/2 |grad1 u|^2): the layout of grad1_u12 in the reference's
 * cutc_int_bh (src/jast_bh.cu:268-303), without its launch-geometry
 * arguments.  Synchronous on the engine stream.
 */
int cutc_jast_bh_dev(int i0, int n1b, int n_grid1, int n_grid2, int n_nuc, int size_bh,
                     const double *r1, const double *r2, const double *rn,
                     const double *c_bh, const int *m_bh, const int *n_bh, const int *o_bh,
                     double a_en, double a_ee, double *grad1u);

/*
 * cutc_jast_bh_dev without any allocation, for callers that cannot let a
 * library allocate device memory: programs whose own memory manager has
 * reserved the whole device (a framework's caching allocator holding all of
 * HBM, where a cudaMalloc from a library fails or fragments that pool), and
 * latency-critical serving loops, where cudaMalloc and cudaFree would stall
 * on device-wide synchronisation.  No counterpart in the reference.
 *
 * Same arguments, layout and results as cutc_jast_bh_dev, plus the stream to
 * run on (NULL = the legacy default stream).  Each call waits for its stream
 * to finish and reads a status word back to the host before it returns.  Its
 * scratch -- per-point nucleus terms, r2 e-n terms and the Jastrow term table,
 * 32 * n1b * n_nuc + 8 * n_grid2 * n_nuc bytes plus ~130 KB -- lives in a
 * fixed 32 MiB device array that every GPU loading this library holds until
 * exit; larger requests are rejected with CUTC_ERR_INVALID and a message
 * before anything runs.  It calls no cudaMalloc, cudaFree or allocating
 * library routine and creates no engine context.  The first call on a device
 * also does the set-up: it looks up the array's device address
 * (cudaGetSymbolAddress, with that device current), so make that first call
 * before any stream capture.  All calls share the one array and each call
 * overwrites what the previous one left there, so calls that overlap on the
 * GPU (different streams or threads) race: serialise them.  Exponents outside
 * [0, 6] and more than 4096 kept terms are found on the device, while the pair
 * kernel runs: the call then returns CUTC_ERR_INVALID with grad1u already
 * overwritten.
 */
int cutc_jast_bh_dev_noalloc(int i0, int n1b, int n_grid1, int n_grid2, int n_nuc, int size_bh,
                             const double *r1, const double *r2, const double *rn,
                             const double *c_bh, const int *m_bh, const int *n_bh,
                             const int *o_bh, double a_en, double a_ee, double *grad1u,
                             void *stream);

/*
 * The failure path of the tensor-core kernels' pipeline waits, checked without a
 * fault: one CTA waits on a barrier that nothing completes, its bounded wait gives
 * up after its limit (2 s), and the call returns CUTC_ERR_TIMEOUT -- the status a
 * build reports when one of its pipeline waits gives up -- with the device still
 * usable.  For tests.  No reference counterpart.
 */
int cutc_check_wait_limit(void);

/*
 * The split-precision contraction alone, on device arrays of the current
 * device: C[m + ldc * n] = sum_k A[m * K + k] * B[n * K + k] for m < M, n < N,
 * with A and B FP64 row-major (K contiguous) and the product formed from
 * n_slices BF16 slices per operand on the tcgen05 tensor cores (3..7 slices).
 * This is the kernel behind CUTC_SPLIT_BF16, exposed for callers that need the
 * GEMM itself.  Synchronous on the engine stream.  No reference counterpart.
 */
int cutc_split_gemm_dev(int n_slices, int M, int N, long long K,
                        const double *A, const double *B, double *C, long long ldc);

/*
 * The plain form's FP64 contraction alone, on device arrays of the current
 * device, with cuBLAS's column-major argument meaning (the reference's
 * cublasDgemm calls, src/build_int2_grad1_u12_ao.cu:152-159 and
 * src/build_int_2e_ao.cu:60-67,97-104, take these operand orders):
 *   C[m + ldc n] = alpha sum_k opA(m, k) B[n ldb + k] + beta C[m + ldc n]
 * for m < M, n < N and each of `batch` problems, whose A, B and C start
 * stride_a, stride_b and stride_c doubles apart.  opA(m, k) = A[m lda + k]
 * when a_kmajor is non-zero (cuBLAS OP_T), else A[k lda + m] (OP_N); B is
 * OP_N.  C is not read when beta == 0.  FP64 DMMA tensor-core tiles; no
 * allocation.  Synchronous on the engine stream.
 */
int cutc_fp64_gemm_dev(int a_kmajor, int M, int N, long long K, double alpha, const double *A,
                       long long lda, long long stride_a, const double *B, long long ldb,
                       long long stride_b, double beta, double *C, long long ldc,
                       long long stride_c, int batch);

/*
 * The launch-geometry check of src/cutc_int.c:79-86 against the current
 * device: block volume > maxThreadsPerBlock or any grid extent > maxGridSize
 * (unsigned comparisons, as the reference's dim3 arithmetic) returns
 * CUTC_ERR_LAUNCH_DIMS (-1).
 */
int cutc_validate_launch_dims(int nxBlocks, int nyBlocks, int nzBlocks,
                              int blockxSize, int blockySize, int blockzSize);

/* ---- serving: continuous batching on one GPU (no reference counterpart) --
 * A server owns n_slots execution contexts (stream, events, workspace) and a
 * worker thread each.  Submitted requests are queued; a free
 * worker takes the first queued request whose device footprint fits the
 * memory budget next to the requests in flight (a request that does not fit
 * runs alone), so requests overlap on the GPU as slots and memory free up.
 * Requests with a non-zero molecule_key keep their molecule arrays (grids,
 * weights, nuclei, AO values) resident in a byte-budgeted LRU cache: a later
 * request with the same key and sizes copies only its Jastrow parameters.
 * All array pointers of a request are host pointers and must stay valid until
 * cutc_server_wait returns for it.  Each result is the same as the one a
 * standalone cutc_int_ex call with the same options gives. */
typedef struct cutc_server cutc_server;

typedef struct cutc_server_config {
    int n_slots;                /* concurrent requests on the GPU (default 4) */
    size_t device_budget_bytes; /* admission budget for requests in flight (0: 3/4 of free) */
    size_t cache_budget_bytes;  /* molecule cache (0: 1/4 of the device budget) */
    size_t tile_budget_bytes;   /* per request: X-tile and int_2e-block working sets, each
                                   (default 8 GiB) */
} cutc_server_config;

typedef struct cutc_request {
    unsigned long long molecule_key; /* 0: no caching; else identifies the molecule arrays */
    int n_grid1, n_grid2, n_ao, n_nuc, size_bh;
    const double *r1, *wr1, *r2, *wr2, *rn, *aos_data1, *aos_data2, *c_bh;
    const int *m_bh, *n_bh, *o_bh;
    double *int2_grad1_u12_ao, *int_2e_ao;
    cutc_options options;       /* device_pointers, stream and max_work_bytes are ignored; an
                                   r1 window is refused */
} cutc_request;

typedef struct cutc_server_stats {
    long completed, failed, queued;
    int in_flight, peak_in_flight;
    long cache_hits, cache_misses;
    size_t cache_bytes;
    double p50_ms, p99_ms, max_ms;  /* submit-to-completion latency of completed requests */
    double builds_per_s;            /* completed / (last completion - first submit) */
} cutc_server_stats;

void cutc_server_default_config(cutc_server_config *cfg);
int cutc_server_create(const cutc_server_config *cfg, cutc_server **server);
int cutc_server_submit(cutc_server *server, const cutc_request *req, unsigned long long *ticket);
/* Blocks until the request is done; returns its status and forgets the ticket. */
int cutc_server_wait(cutc_server *server, unsigned long long ticket, double *latency_ms);
int cutc_server_get_stats(cutc_server *server, cutc_server_stats *stats);
/* Finishes the queued requests, then frees the contexts and the cache. */
void cutc_server_destroy(cutc_server *server);

/* Page-locks (pins) / releases caller host memory, so that outputs written there
 * are copied in directly instead of through the library's pinned staging
 * (cudaHostRegister / cudaHostUnregister).  No reference counterpart. */
int cutc_pin_host(void *ptr, size_t bytes);
int cutc_unpin_host(void *ptr);

/* The device-memory plan of a build, computed on the host (no GPU needed when
 * opt->max_work_bytes is set; with 0 the budget follows the current device's
 * free memory, or is the plan of the engine's last completed build of the same
 * shape, as a build would take it).  The r1 grid is cut into X tiles of
 * tile_rows points; the int_2e contractions run once per block of block_rows
 * points (whole tiles).  Device bytes besides the caller's arrays: fixed_bytes
 * + tile_rows * tile_row_bytes + block_rows * block_row_bytes (+ the molecule
 * arrays for host inputs) = footprint_bytes, which the server admits by.
 * Honours CUTC_TILE_ROWS / CUTC_INT2E_ROWS like cutc_int_ex.  No reference
 * counterpart. */
typedef struct cutc_plan_info {
    int tile_rows, block_rows, n_tiles, n_blocks;
    int slab_cols;              /* int_2e columns per output slab (host outputs) */
    size_t budget_bytes;        /* the budget each of tile and block was sized to */
    size_t fixed_bytes, tile_row_bytes, block_row_bytes, footprint_bytes;
    int x_launches_per_tile;    /* split form: tensor-core launches that share one X
                                   contraction's K (opt->k_split; 0 = automatic) */
} cutc_plan_info;

int cutc_plan(const cutc_options *opt, int n_grid1, int n_grid2, int n_ao, int n_nuc,
              cutc_plan_info *plan);

/* AO values (components = 1) or values and gradients (components = 4) of the
 * basis at n_points points r(3, n_points), written as aos(n_points, n_ao,
 * components) column-major: the layout of aos_data1 / aos_data2.  r and aos are
 * device pointers when device_pointers is 1 (then the call is asynchronous on
 * stream), host pointers otherwise.  No reference counterpart (the reference
 * takes AO values from its caller). */
int cutc_eval_aos(const cutc_basis *basis, int n_points, const double *r, int components,
                  double *aos, int device_pointers, void *stream);

/* X in the MO basis, in the order the reference's cutc_no reads it
 * (src/no_tmpJ_cs_kernel.cu:18-30):
 *   x_mo(g, m, i, j) = sum_{a,b} mo_l_coef(a, i) x_ao(a, b, g, m) mo_r_coef(b, j)
 * x_ao(n_ao, n_ao, n_grid1, components) as cutc_int writes it, mo_l_coef and
 * mo_r_coef (n_ao, n_mo), x_mo(n_grid1, components, n_mo, n_mo), all column-major
 * FP64, components 3 or 4.  Device pointers when device_pointers is 1 (then
 * asynchronous on stream), host pointers otherwise.  No reference counterpart
 * (the reference's workflow does this step outside the library). */
int cutc_x_ao_to_mo(int n_grid1, int n_ao, int n_mo, int components,
                    const double *mo_l_coef, const double *mo_r_coef,
                    const double *x_ao, double *x_mo, int device_pointers, void *stream);

/*
 * The two-electron contraction of the reference's cutc_no (src/cutc_no.c:415-470), on its
 * intermediates: with M = n_mo^2 MO pairs,
 *   no_2e = 1/2 tmpC1^T x_mo + 1/2 tmpC2^T tmpD2,  then no_2e <- no_2e + no_2e^T,
 *   then the (p,q,s,t) -> (p,s,q,t) swap of trans_pqst_psqt_inplace.
 * x_mo is X in the MO basis in cutc_no's order, [(g + n_grid1 m) + 3 n_grid1 (i + n_mo j)]
 * (what cutc_x_ao_to_mo writes); tmpC1 has the same layout (3 n_grid1 x n_mo^2), tmpC2 and
 * tmpD2 are n_grid1 x n_mo^2, no_2e is n_mo^4 (all column-major, FP64).  Options used:
 * precision (plain FP64 as the reference, or the split form: one split contraction over
 * the concatenated K = 4 n_grid1), n_slices, device_pointers, stream.  Synchronous.
 */
int cutc_no_2e(const cutc_options *opt, int n_mo, int n_grid1, const double *tmpC1,
               const double *x_mo, const double *tmpC2, const double *tmpD2, double *no_2e);

/* ---- reference helpers with the reference's names and semantics ------------
 * Device pointers; launched on the legacy default stream without a host
 * synchronisation, as the reference does; errors are recorded for
 * cutc_last_error() (the reference signatures return nothing).
 *
 * trans_inplace (src/add_trans_inplace.cu:25-35): data <- data + data^T for a
 * size x size column-major matrix.
 * trans_pqst_psqt_inplace (src/trans_pqst_psqt_inplace.cu:50-62): the
 * size^4 array data(p,q,s,t) (column-major) becomes data(p,s,q,t).
 * trans_pqst_psqt_copy (src/trans_pqst_psqt_copy.cu:45-57): data_new(p,q,s,t)
 * = data_old(p,s,q,t).  No reference counterpart besides those files. */
void trans_inplace(double *data, int size);
void trans_pqst_psqt_inplace(int size, double *data);
void trans_pqst_psqt_copy(int size, double *data_old, double *data_new);

/* The launch geometry argument of the reference's device-level entry points:
 * the layout of CUDA's dim3 (three unsigned ints), so a caller passing a dim3
 * by value is served unchanged. */
typedef struct cutc_dim3 {
    unsigned int x, y, z;
} cutc_dim3;

/* ---- the reference's device-level stages of cutc_int, under its names ------
 * Same signatures and device-pointer arguments as the reference; the work is
 * ordered on the legacy default stream; failures are recorded for
 * cutc_last_error().  All FP64, a_en = a_ee = 1 as in the reference.
 *
 * cutc_int_bh (src/jast_bh.cu:268-303): the pair terms of r1 points
 * [ii0, ii0 + n_grid1_eff) against r2 points [jj0, jj0 + n_grid2_eff), written
 * to grad1_u12[c * n_grid1_tot * n_grid2_tot + i * n_grid2_tot + j] with c = 0..2
 * the gradient and c = 3 -1/2 |grad1 u|^2.  dimGrid / dimBlock are validated
 * like cutc_int's launch integers and otherwise ignored.  Returns when done.
 *
 * int_long_range (src/long_range_integ.cu:52-67):
 * out[j + n_grid2_tot (b + n_ao a)] = wr2[jj0 + j] chi_a chi_b at r2 point
 * jj0 + j, for j < n_grid2_eff; aos_data2 is (n_grid2, n_ao[, 4]).
 * int_short_range_herm (src/short_range_integ_herm.cu:51-64):
 * out[g + n_grid1 (b + n_ao a)] = wr1 chi_a chi_b.
 * int_short_range_nonherm (src/short_range_integ_nonherm.cu:69-82):
 * out[g + n_grid1 m + 3 n_grid1 (b + n_ao a)] = wr1 (chi_b d_m chi_a - chi_a d_m chi_b).
 * These three are asynchronous, like the reference's.
 *
 * get_int2_grad1_u12_ao (src/build_int2_grad1_u12_ao.cu:9-347): X with all four
 * components, int2_grad1_u12_ao(n_ao, n_ao, n_grid1, 4) column-major on the
 * device; the streamed X build of cutc_int_ex (plain FP64, or the split form
 * with CUTC_PRECISION=split).  Returns when done.
 * get_int_2e_ao (src/build_int_2e_ao.cu:11-145): int_2e_ao = A + A^T with
 * A = X_3 S0 - 1/2 sum_m X_m S_m from the caller's int2_grad1_u12(n_ao, n_ao,
 * n_grid1, 4), in FP64.  Returns when done. */
void cutc_int_bh(cutc_dim3 dimGrid, cutc_dim3 dimBlock,
                 int ii0, int n_grid1_eff, int n_grid1_tot,
                 int jj0, int n_grid2_eff, int n_grid2_tot,
                 int n_nuc, int size_bh,
                 double *r1, double *r2, double *rn,
                 double *c_bh, int *m_bh, int *n_bh, int *o_bh,
                 double *grad1_u12);
void int_long_range(int jj0, int n_grid2_eff, int n_grid2_tot,
                    int n_grid2, int n_ao, double *wr2, double *aos_data2,
                    double *int_fct_long_range);
void int_short_range_herm(int n_grid1, int n_ao, double *wr1, double *aos_data1,
                          double *int_fct_short_range_herm);
void int_short_range_nonherm(int n_grid1, int n_ao, double *wr1, double *aos_data1,
                             double *int_fct_short_range_nonherm);
void get_int2_grad1_u12_ao(cutc_dim3 dimGrid, cutc_dim3 dimBlock,
                           int n_grid1, int n_grid2, int n_ao, int n_nuc, int size_bh,
                           double *r1, double *r2, double *wr2, double *rn, double *aos_data2,
                           double *c_bh, int *m_bh, int *n_bh, int *o_bh,
                           double *int2_grad1_u12_ao);
void get_int_2e_ao(int n_grid1, int n_ao, double *wr1, double *aos_data1,
                   double *int2_grad1_u12, double *int_2e_ao);

/* Message describing the last non-zero status returned on this thread. */
const char *cutc_last_error(void);

/* Frees the engine's cached device workspace on the current device. */
void cutc_release(void);

#ifdef __cplusplus
}
#endif

#endif
