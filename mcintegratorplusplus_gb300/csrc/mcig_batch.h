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

// one estimator series: n values at data[i * stride]
struct BatchSeries {
    const double *data;
    int64_t n, stride;
    int one_d, noop;
};

void mcig_batch_launch(const KParams *cfg, const BatchPhase *ph, const int2 *units, int nunits, int *counter, int grid,
                       int block, cudaStream_t st);
void mcig_batch_estimate_launch(const BatchSeries *series, int nseries, double *avg, double *err, cudaStream_t st);
