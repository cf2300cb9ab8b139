// Persistent batched sampling kernel: many independent integrals (each its own
// KParams: dimension, sampling functions, move, observables, seed) in one launch
// per ndim bucket.  Each warp takes 32 consecutive work units (integral, chain)
// from an atomic queue sorted longest-first, and each lane runs the whole of
// MCI::integrate for its chain: findMRT2Step, burn-in and sampling with the
// accumulators (reference src/MCIntegrator.cpp:43-82), with the general float
// kernel's code (mcig_generic.cuh), so a chain gives the same numbers here as
// in an individual launch of the general kernel.
#include "mcig_generic.cuh"
#include "mcig_batch.h"

__global__ void __launch_bounds__(256) mcig_batch_kernel(const KParams *__restrict__ cfg, const BatchPhase *__restrict__ ph,
                                                         const int2 *__restrict__ units, int nunits, int *counter)
{
    const int lane = threadIdx.x & 31;
    while (true) {
        int base = 0;
        if (lane == 0) { base = atomicAdd(counter, 32); }
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= nunits) { break; }
        const int u = base + lane;
        if (u < nunits) {
            const int2 w = units[u];
            const KParams &p = cfg[w.x];
            const BatchPhase &q = ph[w.x];
            GenericSampler<float, RNG_PHILOX, true> s(p, w.y, p.fblob);
            if (q.do_find) { s.run_calibration(q.movetype, q.min_stat); }
            if (q.ndecorr > 0) { s.run_steps(q.movetype, q.ndecorr); }
            s.run_sample(q.movetype, p.nsteps);
            s.store_state();
        }
    }
}

void mcig_batch_launch(const KParams *cfg, const BatchPhase *ph, const int2 *units, int nunits, int *counter, int grid,
                       int block, cudaStream_t st)
{
    mcig_batch_kernel<<<grid, block, 0, st>>>(cfg, ph, units, nunits, counter);
}
