// Register-resident float sampling kernels, all-coordinate move, up to 16 dimensions
// (mcig_fast.cuh).  At 17..32 dimensions the register-resident kernels exist for a single
// sampling function of one kind (sample_fast_pk32*.cu); other 32-D configurations run
// the general kernel (a 32-D kernel over every sampling-function kind took over five
// minutes to compile).
#include "mcig_fast.cuh"
#include "mcig_launchers.h"

mcig_launch_fn mcig_fast_launcher_vec(int kahan, int maxd);
mcig_launch_fn mcig_fast_launcher_pk16(int kahan, int pk, int moments);
mcig_launch_fn mcig_fast_launcher_pk16_lean1(int kahan, int pk, int moments);
mcig_launch_fn mcig_fast_launcher_pk16_lean2(int kahan, int pk, int moments);
mcig_launch_fn mcig_fast_launcher_pk32(int kahan, int pk);

static mcig_launch_fn launcher_all(int kahan, int maxd)
{
    switch (maxd) {
    case 4: return kahan ? mcig_fast_launch<4, MCIG_MOVE_ALL, true> : mcig_fast_launch<4, MCIG_MOVE_ALL, false>;
    case 8: return kahan ? mcig_fast_launch<8, MCIG_MOVE_ALL, true> : mcig_fast_launch<8, MCIG_MOVE_ALL, false>;
    case 16: return kahan ? mcig_fast_launch<16, MCIG_MOVE_ALL, true> : mcig_fast_launch<16, MCIG_MOVE_ALL, false>;
    default: return nullptr;
    }
}

mcig_launch_fn mcig_fast_launcher(int kahan, int move, int maxd, int pk, int moments, int lean)
{
    if (move == MCIG_MOVE_ALL && maxd == 16 && lean) { // one step-size type, unbound domain, known draws
        mcig_launch_fn f = lean == 2 ? mcig_fast_launcher_pk16_lean2(kahan, pk, moments) : mcig_fast_launcher_pk16_lean1(kahan, pk, moments);
        if (f) { return f; }
    }
    if (move == MCIG_MOVE_ALL && pk != PK_ANY) { // one-pdf kernels where they exist
        mcig_launch_fn f = maxd == 16 ? mcig_fast_launcher_pk16(kahan, pk, moments) : (maxd == 32 ? mcig_fast_launcher_pk32(kahan, pk) : nullptr);
        if (f) { return f; }
    }
    if (move == MCIG_MOVE_ALL) { return launcher_all(kahan, maxd); }
    if (move == MCIG_MOVE_VEC) { return mcig_fast_launcher_vec(kahan, maxd); }
    return nullptr;
}
