// Float sampling kernels with two lanes per chain for one precision-matrix or exp(-x.x)
// sampling function in 9..16 coordinates (mcig_pair.cuh), Kahan float or double block sums.
#include "mcig_pair.cuh"
#include "mcig_launchers.h"

mcig_launch_fn mcig_pair_launcher(int kahan, int pk, int moments)
{
    if (moments) { // observables x and x.x only
        switch (pk) {
        case PK_GAUSS: return kahan ? mcig_pair_launch<PK_GAUSS, true, true> : mcig_pair_launch<PK_GAUSS, false, true>;
        case PK_PREC: return kahan ? mcig_pair_launch<PK_PREC, true, true> : mcig_pair_launch<PK_PREC, false, true>;
        default: return nullptr;
        }
    }
    switch (pk) {
    case PK_GAUSS: return kahan ? mcig_pair_launch<PK_GAUSS, true> : mcig_pair_launch<PK_GAUSS, false>;
    case PK_PREC: return kahan ? mcig_pair_launch<PK_PREC, true> : mcig_pair_launch<PK_PREC, false>;
    default: return nullptr;
    }
}
