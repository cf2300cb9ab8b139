// General sampling kernel, float arithmetic with log-space acceptance, Philox
// draws; accumulator sums in double.
#include "mcig_generic.cuh"
#include "mcig_launchers.h"

static void launch_f32_acc64(const KParams &p, const FastConst *, int movetype, int grid, int block, size_t smem,
                           cudaStream_t st)
{
    auto k = mcig_generic_kernel<float, RNG_PHILOX, false>;
    if (smem > 48 * 1024) { cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); }
    k<<<grid, block, smem, st>>>(p, movetype);
}

mcig_launch_fn mcig_generic_launcher_f32_acc64() { return launch_f32_acc64; }
