// Register-resident float sampling kernels, single-vector move, up to 16
// dimensions (mcig_fast.cuh); larger walkers use the general kernel.
#include "mcig_fast.cuh"
#include "mcig_launchers.h"

mcig_launch_fn mcig_fast_launcher_vec(int kahan, int maxd)
{
    switch (maxd) {
    case 4: return kahan ? mcig_fast_launch<4, MCIG_MOVE_VEC, true> : mcig_fast_launch<4, MCIG_MOVE_VEC, false>;
    case 8: return kahan ? mcig_fast_launch<8, MCIG_MOVE_VEC, true> : mcig_fast_launch<8, MCIG_MOVE_VEC, false>;
    case 16: return kahan ? mcig_fast_launch<16, MCIG_MOVE_VEC, true> : mcig_fast_launch<16, MCIG_MOVE_VEC, false>;
    default: return nullptr;
    }
}
