// Float sampling kernels with several lanes per chain for one mixture sampling function
// (mcig_lanes.cuh): 32-coordinate walkers on 4 or 8 lanes, Kahan float or double block sums.
#include "mcig_lanes.cuh"
#include "mcig_launchers.h"

mcig_launch_fn mcig_lanes_launcher(int kahan, int maxd, int lpc)
{
    if (maxd != 32) { return nullptr; }
    switch (lpc) {
    case 4: return kahan ? mcig_lanes_launch<32, 4, true> : mcig_lanes_launch<32, 4, false>;
    case 8: return kahan ? mcig_lanes_launch<32, 8, true> : mcig_lanes_launch<32, 8, false>;
    default: return nullptr;
    }
}
