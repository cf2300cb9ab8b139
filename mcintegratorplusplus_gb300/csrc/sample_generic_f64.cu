// General sampling kernel, double arithmetic in the reference's operation order
// (this unit is compiled with -fmad=false), Philox or replayed draws.
#include "mcig_generic.cuh"
#include "mcig_launchers.h"

template <class R, int RNG, bool KAHAN>
static void launch_generic(const KParams &p, const FastConst *, int movetype, int grid, int block, size_t smem,
                           cudaStream_t st)
{
    auto k = mcig_generic_kernel<R, RNG, KAHAN>;
    if (smem > 48 * 1024) { cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); }
    k<<<grid, block, smem, st>>>(p, movetype);
}

mcig_launch_fn mcig_generic_launcher_f32(int precision);

mcig_launch_fn mcig_generic_launcher(int precision, int rng)
{
    if (precision == MCIG_PREC_FP64) {
        return rng == RNG_TAPE ? launch_generic<double, RNG_TAPE, false> : launch_generic<double, RNG_PHILOX, false>;
    }
    if (rng != RNG_PHILOX) { return nullptr; }
    return mcig_generic_launcher_f32(precision);
}
