// Register-resident float sampling kernels for one-pdf configurations, all-coordinate
// move, 32 dimensions, double block sums (mcig_fast.cuh, PK_GAUSS / PK_MIX); a unit of its
// own for compile time.
#include "mcig_fast.cuh"
#include "mcig_launchers.h"

mcig_launch_fn mcig_fast_launcher_pk32d(int pk)
{
    switch (pk) {
    case PK_GAUSS: return mcig_fast_launch<32, MCIG_MOVE_ALL, false, PK_GAUSS>;
    case PK_MIX: return mcig_fast_launch<32, MCIG_MOVE_ALL, false, PK_MIX>;
    default: return nullptr;
    }
}
