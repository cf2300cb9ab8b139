// Register-resident float sampling kernels for a single 32-D precision-matrix sampling
// function, all-coordinate move, Kahan float or double block sums (mcig_fast.cuh,
// PK_PREC); a unit of its own for compile time.
#include "mcig_fast.cuh"
#include "mcig_launchers.h"

mcig_launch_fn mcig_fast_launcher_pk32p(int kahan)
{
    return kahan ? mcig_fast_launch<32, MCIG_MOVE_ALL, true, PK_PREC> : mcig_fast_launch<32, MCIG_MOVE_ALL, false, PK_PREC>;
}
