// Float sampling kernels with several lanes per chain for one mixture sampling function
// (mcig_lanes.cuh): 32-coordinate walkers on 4 or 8 lanes, Kahan float or double block sums,
// uniform or Gaussian move draws.
#include "mcig_lanes.cuh"
#include "mcig_launchers.h"

template <int LPC, bool GAUSS>
static mcig_launch_fn pick(int kahan)
{
    return kahan ? mcig_lanes_launch<32, LPC, true, GAUSS> : mcig_lanes_launch<32, LPC, false, GAUSS>;
}

mcig_launch_fn mcig_lanes_launcher(int kahan, int maxd, int lpc, int gauss)
{
    if (maxd != 32) { return nullptr; }
    switch (lpc) {
    case 4: return gauss ? pick<4, true>(kahan) : pick<4, false>(kahan);
    case 8: return gauss ? pick<8, true>(kahan) : pick<8, false>(kahan);
    default: return nullptr;
    }
}
