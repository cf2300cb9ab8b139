// Register-resident float sampling kernels for one-pdf configurations, all-coordinate
// move, 32 dimensions, Kahan float block sums (mcig_fast.cuh, PK_*); the precision-matrix
// kernels are in sample_fast_pk32p.cu (units of their own for compile time).
#include "mcig_fast.cuh"
#include "mcig_launchers.h"

mcig_launch_fn mcig_fast_launcher_pk32d(int pk);
mcig_launch_fn mcig_fast_launcher_pk32p(int kahan);

mcig_launch_fn mcig_fast_launcher_pk32(int kahan, int pk)
{
    if (pk == PK_PREC) { return mcig_fast_launcher_pk32p(kahan); }
    if (!kahan) { return mcig_fast_launcher_pk32d(pk); }
    switch (pk) {
    case PK_GAUSS: return mcig_fast_launch<32, MCIG_MOVE_ALL, true, PK_GAUSS>;
    case PK_MIX: return mcig_fast_launch<32, MCIG_MOVE_ALL, true, PK_MIX>;
    default: return nullptr;
    }
}
