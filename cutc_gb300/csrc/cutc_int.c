/*
 * cutc_int: the drop-in entry point, compiled as C like the reference's
 * driver (src/cutc_int.c:15-243, built by gcc in the reference Makefile:57-62).
 *
 * Same argument list, layouts and return codes as the reference.  The launch
 * integers are validated like src/cutc_int.c:79-86 and then ignored.  The
 * precision form is plain FP64 unless the environment variable
 * CUTC_PRECISION=split selects the BF16-slice form, so an unmodified Fortran
 * or C caller can opt in without code changes.  CUTC_SLICES (3..7, default 5)
 * sets that form's slice count: 6 reaches the plain form's error class.
 */
#include <stdlib.h>
#include <string.h>

#include "cutc_int.h"

int cutc_int(int nxBlocks, int nyBlocks, int nzBlocks,
             int blockxSize, int blockySize, int blockzSize,
             int n_grid1, int n_grid2, int n_ao, int n_nuc, int size_bh,
             double *r1, double *wr1, double *r2, double *wr2, double *rn,
             double *aos_data1, double *aos_data2,
             double *c_bh, int *m_bh, int *n_bh, int *o_bh,
             double *int2_grad1_u12_ao, double *int_2e_ao)
{
    int s = cutc_validate_launch_dims(nxBlocks, nyBlocks, nzBlocks,
                                      blockxSize, blockySize, blockzSize);
    if (s != CUTC_OK)
        return s;
    cutc_options opt;
    cutc_default_options(&opt);
    const char *prec = getenv("CUTC_PRECISION");
    if (prec && strcmp(prec, "split") == 0) {
        opt.precision = CUTC_SPLIT_BF16;
        const char *sl = getenv("CUTC_SLICES");
        if (sl && *sl) {
            char *end = NULL;
            const long v = strtol(sl, &end, 10);
            /* a malformed or out-of-range count reaches cutc_int_ex, which refuses it */
            opt.n_slices = (*end == '\0' && v >= 0 && v <= 64) ? (int)v : -1;
        }
    }
    return cutc_int_ex(&opt, n_grid1, n_grid2, n_ao, n_nuc, size_bh,
                       r1, wr1, r2, wr2, rn, aos_data1, aos_data2,
                       c_bh, m_bh, n_bh, o_bh, int2_grad1_u12_ao, int_2e_ao, NULL);
}
