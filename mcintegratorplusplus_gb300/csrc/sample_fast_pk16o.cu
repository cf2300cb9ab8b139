// Register-resident float sampling kernels for one exp(-x.x) or precision-matrix sampling
// function, all-coordinate move with one step-size type, up to 16 dimensions (mcig_fast.cuh,
// ONET), with the general observable code or the x / x.x variant (MOMENTS), Kahan float or
// double block sums.  A unit of its own, so the parallel build compiles it beside
// sample_fast_pk16.cu.
#include "mcig_fast.cuh"
#include "mcig_launchers.h"

template <int PK>
static mcig_launch_fn pick(int kahan, int moments)
{
    if (moments) {
        return kahan ? mcig_fast_launch<16, MCIG_MOVE_ALL, true, PK, true, true> : mcig_fast_launch<16, MCIG_MOVE_ALL, false, PK, true, true>;
    }
    return kahan ? mcig_fast_launch<16, MCIG_MOVE_ALL, true, PK, false, true> : mcig_fast_launch<16, MCIG_MOVE_ALL, false, PK, false, true>;
}

mcig_launch_fn mcig_fast_launcher_pk16_onetype(int kahan, int pk, int moments)
{
    switch (pk) {
    case PK_GAUSS: return pick<PK_GAUSS>(kahan, moments);
    case PK_PREC: return pick<PK_PREC>(kahan, moments);
    default: return nullptr;
    }
}
