// General sampling kernel, float arithmetic with log-space acceptance, Philox
// draws; accumulator sums in float with Kahan compensation.
#include "mcig_generic.cuh"
#include "mcig_launchers.h"

static void launch_f32_kahan(const KParams &p, const FastConst *, int movetype, int grid, int block, size_t smem,
                           cudaStream_t st)
{
    auto k = mcig_generic_kernel<float, RNG_PHILOX, true>;
    if (smem > 48 * 1024) { cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); }
    k<<<grid, block, smem, st>>>(p, movetype);
}

mcig_launch_fn mcig_generic_launcher_f32_acc64();

mcig_launch_fn mcig_generic_launcher_f32(int precision)
{
    return precision == MCIG_PREC_FP32 ? launch_f32_kahan : mcig_generic_launcher_f32_acc64();
}
