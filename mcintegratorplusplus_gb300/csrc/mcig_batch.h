// mcig_batch.h -- types and launchers of the batched integration (sample_batch.cu).
#pragma once
#include <cuda_runtime.h>
#include "mcig_common.cuh"

// per integral: the phases of MCI::integrate run before sampling
struct BatchPhase {
    int64_t min_stat; // findMRT2Step steps per iteration
    int64_t ndecorr;  // burn-in steps (0: none)
    int do_find;
    int movetype;
};

// one work item of the persistent launch: `count` (<= 32) chains, one per lane of the warp
// that takes it (their integrals and indices in the task's BatchLane entries; `integral` and
// `chain0` name the first); `variant`, common to them, selects the code:
// 0 the general sampler, 1 + u (uniform sub-moves) or 4 + u (Gaussian sub-moves) the
// block-separable sampler with its sub-step loop unrolled 2^u times
struct BatchTask {
    int integral;
    int chain0;
    int count;
    int variant;
};

// the chain a lane of a task runs: tasks pack up to 32 chains of possibly different integrals
// of the same code variant (BatchTask::integral / chain0 then name the first), so that
// integrals with fewer than 32 chains do not leave a warp's other lanes idle
struct BatchLane {
    int integral;
    int chain;
};

#define MCIG_BS_MAXR 4   // sums of x_i^2 over coordinate ranges kept by the block-separable sampler
#define MCIG_BS_MAXNS 8  // MultiStepMove sub-steps of the block-separable sampler
#define MCIG_BS_MAXOBS 4 // observables of the block-separable sampler
#define MCIG_BS_MAXV 16  // observable values of the block-separable sampler

// Block-separable configuration of an integral (host-made): every sampling function and
// every MultiStepMove sub-pdf is an isotropic Gaussian factor exp(-c sum_{a<=i<b} x_i^2)
// over a coordinate range, so the log densities are sums over the ranges' sums of squares
// S_r; pc[r] (sc[r]) is the sum of the coefficients c of the sampling functions (sub-pdfs)
// over range r.  Observables read the sums: value j of observable o is S[orng[o] + j].
// The ranges of the sampling functions, the sub-pdfs and the observables must coincide and
// number at most MCIG_BS_MAXR (the uneven-batch form: 2-4 factors, x.x per factor).
struct BatchSep {
    int nr;
    int ra[MCIG_BS_MAXR], rb[MCIG_BS_MAXR];
    float pc[MCIG_BS_MAXR], sc[MCIG_BS_MAXR];
    int orng[MCIG_BS_MAXOBS];
};

// one estimator series: n values at data[i * stride]
struct BatchSeries {
    const double *data;
    int64_t n, stride;
    int one_d, noop;
};

// prec MCIG_PREC_*, rng RNG_PHILOX / RNG_TAPE (tape: FP64); walk, nslot, nundo: the
// block-separable sampler's shared memory per lane (largest ndim, observable values and
// MultiStepMove sub-steps of its integrals)
void mcig_batch_launch(int prec, int rng, const KParams *cfg, const BatchPhase *ph, const BatchSep *sep,
                       const BatchTask *tasks, const BatchLane *lanes, int ntasks, int *counter, int grid, int block,
                       int walk, int nslot, int nundo, cudaStream_t st);
// resident blocks per SM of the launch at this block size, for sizing the persistent grid
int mcig_batch_blocks_per_sm(int prec, int rng, int block, int walk, int nslot, int nundo);
void mcig_batch_estimate_launch(const BatchSeries *series, int nseries, double *avg, double *err, cudaStream_t st);
