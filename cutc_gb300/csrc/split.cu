// Split-precision (BF16-slice) contractions on tcgen05.
#include "common.cuh"
#include "split.cuh"

namespace cutc {

size_t split_r1_row_bytes(const Request &) { return 0; }

static int not_built()
{
    cutc_set_error(CUTC_ERR_INVALID, "the split-precision form is not available in this build");
    return CUTC_ERR_INVALID;
}

int split_prepare_x(Engine *, const Request &, cudaStream_t, const double *, const double *,
                    int64_t, int, SplitPlan &)
{
    return not_built();
}

int split_x_tile(Engine *, const Request &, cudaStream_t, SplitPlan &, const double *, int, int,
                 double *)
{
    return not_built();
}

int split_int2e(Engine *, const Request &, cudaStream_t, SplitPlan &, const double *,
                const double *, const double *, double *)
{
    return not_built();
}

}  // namespace cutc
