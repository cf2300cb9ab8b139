// Register-resident float sampling kernel, all-coordinate move, 32 dimensions,
// double block sums (mcig_fast.cuh); a unit of its own for compile time.
#include "mcig_fast.cuh"
#include "mcig_launchers.h"

mcig_launch_fn mcig_fast_launcher_all32d() { return mcig_fast_launch<32, MCIG_MOVE_ALL, false>; }
