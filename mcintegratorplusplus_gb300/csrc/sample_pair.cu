// Float sampling kernels with two lanes per chain for one precision-matrix or exp(-x.x)
// sampling function in 9..16 coordinates (mcig_pair.cuh): Kahan float or double block sums,
// the general observable code or the x / x.x variant, uniform or Gaussian move draws.
#include "mcig_pair.cuh"
#include "mcig_launchers.h"

template <int PK, bool MOMENTS, bool GAUSS>
static mcig_launch_fn pick(int kahan)
{
    return kahan ? mcig_pair_launch<PK, true, MOMENTS, GAUSS> : mcig_pair_launch<PK, false, MOMENTS, GAUSS>;
}

template <int PK>
static mcig_launch_fn pick_pk(int kahan, int moments, int gauss)
{
    if (moments) { return gauss ? pick<PK, true, true>(kahan) : pick<PK, true, false>(kahan); }
    return gauss ? pick<PK, false, true>(kahan) : pick<PK, false, false>(kahan);
}

mcig_launch_fn mcig_pair_launcher(int kahan, int pk, int moments, int gauss)
{
    switch (pk) {
    case PK_GAUSS: return pick_pk<PK_GAUSS>(kahan, moments, gauss);
    case PK_PREC: return pick_pk<PK_PREC>(kahan, moments, gauss);
    default: return nullptr;
    }
}
