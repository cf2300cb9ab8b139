// Register-resident float sampling kernels, all-coordinate move (mcig_fast.cuh).
#include "mcig_fast.cuh"
#include "mcig_launchers.h"

mcig_launch_fn mcig_fast_launcher_all(int kahan, int maxd)
{
    switch (maxd) {
    case 4: return kahan ? mcig_fast_launch<4, MCIG_MOVE_ALL, true> : mcig_fast_launch<4, MCIG_MOVE_ALL, false>;
    case 8: return kahan ? mcig_fast_launch<8, MCIG_MOVE_ALL, true> : mcig_fast_launch<8, MCIG_MOVE_ALL, false>;
    case 16: return kahan ? mcig_fast_launch<16, MCIG_MOVE_ALL, true> : mcig_fast_launch<16, MCIG_MOVE_ALL, false>;
    case 32: return kahan ? mcig_fast_launch<32, MCIG_MOVE_ALL, true> : mcig_fast_launch<32, MCIG_MOVE_ALL, false>;
    default: return nullptr;
    }
}

mcig_launch_fn mcig_fast_launcher_vec(int kahan, int maxd);

mcig_launch_fn mcig_fast_launcher(int kahan, int move, int maxd)
{
    if (move == MCIG_MOVE_ALL) { return mcig_fast_launcher_all(kahan, maxd); }
    if (move == MCIG_MOVE_VEC) { return mcig_fast_launcher_vec(kahan, maxd); }
    return nullptr;
}
