// Engine context, workspace and request description (host side).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "cutc_int.h"

namespace cutc {

constexpr int kNumEvents = 12;

// Grow-only pinned host buffers: outputs bound for pageable caller memory leave
// the device through them.
struct PinnedPool {
    struct Buf {
        void *p = nullptr;
        size_t cap = 0;
    };
    Buf bufs[4];
    int get(int k, size_t bytes, void **out);
    void release();
};

// Grow-only device buffers, one per slot, reused across calls.
//
// The default plan of a build (r1 rows per tile and per int_2e block) is sized from the
// device's free memory, which the buffers kept from the previous build no longer count
// in.  So the workspace remembers the plan of its last completed default-budget build
// with its shape (the fields that set the buffer sizes): a build of the same shape takes
// that plan again, reusing every buffer at its size.  Repeated builds of a molecule then
// tile r1 alike (same bits in the split form, whose int_2e row scales are per block)
// however much memory the first build left held.
struct PlanMemo {
    uint64_t key = 0;   // 0: none
    uint64_t path = 0;  // the pair-term path of that build (its other buffers)
    size_t budget = 0;
    int64_t n1t = 0, kb = 0;
};
struct Workspace {
    struct Buf {
        void *p = nullptr;
        size_t cap = 0;
    };
    std::vector<Buf> bufs;
    int get(int slot, size_t bytes, void **out);
    void release();
    // the remembered plan (readable from any thread)
    bool recall(uint64_t key, PlanMemo *out);
    void remember(const PlanMemo &m);

  private:
    std::mutex memo_mu;
    PlanMemo memo;
};

struct Engine {
    int device = 0;
    int n_sm = 0;
    int max_threads_per_block = 1024;
    int max_grid[3] = {0, 0, 0};
    cudaStream_t stream = nullptr;
    cudaStream_t xfer = nullptr;  // device-to-host copies of finished r1 tiles
    cudaEvent_t ev[kNumEvents];
    std::vector<cudaEvent_t> tile_ev;  // per-tile timing events (grown on demand)
    Workspace ws;
    PinnedPool pinned;
    // Molecule-dependent operands left in the workspace by the previous build:
    // (molecule tag, buffer address) of the X-build A operand and of the int_2e
    // B operands.  A build with the same non-zero tag and the same buffer skips
    // rebuilding them.
    uint64_t tag_x = 0, tag_i = 0;
    const void *tag_x_buf = nullptr, *tag_i_buf = nullptr;
    std::mutex mu;
};

// One integral build, in the reference's argument layout.
struct Request {
    int precision = CUTC_PLAIN_FP64;
    int n_slices = 5;
    double a_en = 1.0, a_ee = 1.0;
    int x_components = 3;
    int device_pointers = 0;  // every array on the device
    int in_device = 0;        // molecule arrays (r1 .. aos2) on the device
    int out_device = 0;       // X and int_2e on the device
    size_t max_work_bytes = 0;
    int tile_rows = 0;  // optional cap on r1 rows per X tile
    int int2e_rows = 0; // optional cap on r1 rows per int_2e block
    int pair_fp64 = 0;  // split form: FP64 pair terms
    int k_split = 0;    // split form: max K per tensor-core launch (0 = default)
    int int2e_layout = CUTC_INT2E_PQST;
    const cutc_basis *basis = nullptr;  // evaluates aos1 / aos2 when those are NULL
    uint64_t mol_tag = 0;  // non-zero: molecule arrays identical to earlier builds with this tag
    int x_only = 0;        // X alone (int_2e output NULL): wr1, aos1 and I are not used
    int i_only = 0;        // int_2e alone (X output NULL): X is formed but not returned
    cudaStream_t stream = nullptr;
    int n1 = 0, n2 = 0, nA = 0, nN = 0, nB = 0;
    int64_t ld1 = 0;  // leading dimension (points) of aos1 when it is a window of a larger grid
                      // (0: n1)
    const double *r1 = nullptr, *wr1 = nullptr, *r2 = nullptr, *wr2 = nullptr, *rn = nullptr;
    const double *aos1 = nullptr, *aos2 = nullptr;
    const double *c_bh = nullptr;
    const int *m_bh = nullptr, *n_bh = nullptr, *o_bh = nullptr;
    double *X = nullptr, *I = nullptr;
};

int get_engine(Engine **out);
// A private execution context (streams, events, workspace) on device dev.
int make_engine(int dev, Engine **out);
void destroy_engine(Engine *E);
// Device bytes one build needs besides its molecule arrays, for a given r1-tile budget.
size_t build_footprint(const Request &R, size_t tile_budget);
int build_terms(const Request &R, std::vector<double> &coef, std::vector<int> &exps,
                std::vector<int> &off);
int run_build(Engine *E, const Request &R, cutc_stats *stats);
// FP64 pair terms on device arrays: r1 rows [i0, i0 + n1b) (of n1) against r2 points
// [j0, j0 + n2b), written to G[c * plane + i * ldg + j]; synchronous on st.
int run_pair_only(Engine *E, cudaStream_t st, int i0, int n1b, int n1, int j0, int n2b,
                  int64_t ldg, int64_t plane, int nN, int nB, const double *r1, const double *r2,
                  const double *rn, const double *c_bh, const int *m_bh, const int *n_bh,
                  const int *o_bh, double a_en, double a_ee, double *G);
void note_launches(int n);
long launches_so_far();

}  // namespace cutc
