// Register-resident float sampling kernels for one exp(-x.x) or precision-matrix sampling
// function, all-coordinate move with one step-size type and uniform draws, unbound domain, up to 16
// dimensions (mcig_fast.cuh, LEAN = 1), with the general observable code or the x / x.x
// variant (MOMENTS, also with one observable in each of its four groups: FIXED4), Kahan float
// or double block sums.  Units of their own, so the parallel
// build compiles them beside sample_fast_pk16.cu.
#include "mcig_fast.cuh"
#include "mcig_launchers.h"

template <int PK>
static mcig_launch_fn pick(int kahan, int moments)
{
    if (moments == 2) { // one observable in each group, nskip 1, ndim 16
        return kahan ? mcig_fast_launch<16, MCIG_MOVE_ALL, true, PK, true, 1, true> : mcig_fast_launch<16, MCIG_MOVE_ALL, false, PK, true, 1, true>;
    }
    if (moments) {
        return kahan ? mcig_fast_launch<16, MCIG_MOVE_ALL, true, PK, true, 1> : mcig_fast_launch<16, MCIG_MOVE_ALL, false, PK, true, 1>;
    }
    return kahan ? mcig_fast_launch<16, MCIG_MOVE_ALL, true, PK, false, 1> : mcig_fast_launch<16, MCIG_MOVE_ALL, false, PK, false, 1>;
}

mcig_launch_fn mcig_fast_launcher_pk16_lean1(int kahan, int pk, int moments)
{
    switch (pk) {
    case PK_GAUSS: return pick<PK_GAUSS>(kahan, moments);
    case PK_PREC: return pick<PK_PREC>(kahan, moments);
    default: return nullptr;
    }
}
