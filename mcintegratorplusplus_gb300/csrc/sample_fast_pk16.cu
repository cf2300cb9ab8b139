// Register-resident float sampling kernels for one-pdf configurations, all-coordinate
// move, up to 16 dimensions: the log density is straight-line code for its kind
// (mcig_fast.cuh, PK_*), with Kahan float or double block sums.
#include "mcig_calib.cuh"
#include "mcig_launchers.h"

mcig_launch_fn mcig_fast_launcher_pk16(int kahan, int pk, int moments)
{
    if (moments) { // observables x and x.x only (FastSampler's MOMENTS)
        switch (pk) {
        case PK_GAUSS:
            return kahan ? mcig_fast_launch<16, MCIG_MOVE_ALL, true, PK_GAUSS, true> : mcig_fast_launch<16, MCIG_MOVE_ALL, false, PK_GAUSS, true>;
        case PK_PREC:
            return kahan ? mcig_fast_launch<16, MCIG_MOVE_ALL, true, PK_PREC, true> : mcig_fast_launch<16, MCIG_MOVE_ALL, false, PK_PREC, true>;
        default: break;
        }
    }
    switch (pk) {
    case PK_GAUSS: return kahan ? mcig_fast_launch<16, MCIG_MOVE_ALL, true, PK_GAUSS> : mcig_fast_launch<16, MCIG_MOVE_ALL, false, PK_GAUSS>;
    case PK_PREC: return kahan ? mcig_fast_launch<16, MCIG_MOVE_ALL, true, PK_PREC> : mcig_fast_launch<16, MCIG_MOVE_ALL, false, PK_PREC>;
    case PK_MIX: return kahan ? mcig_fast_launch<16, MCIG_MOVE_ALL, true, PK_MIX> : mcig_fast_launch<16, MCIG_MOVE_ALL, false, PK_MIX>;
    default: return nullptr;
    }
}

// calibration with the split tail (mcig_calib.cuh) for one exp(-x.x) or precision-matrix
// sampling function and uniform (gauss 0) or Gaussian (1) draws; NULL for other kinds
mcig_launch_fn mcig_calib_launcher_pk16(int pk, int gauss)
{
    switch (pk) {
    case PK_GAUSS: return gauss ? mcig_calib_launch<16, PK_GAUSS, 2> : mcig_calib_launch<16, PK_GAUSS, 1>;
    case PK_PREC: return gauss ? mcig_calib_launch<16, PK_PREC, 2> : mcig_calib_launch<16, PK_PREC, 1>;
    default: return nullptr;
    }
}
