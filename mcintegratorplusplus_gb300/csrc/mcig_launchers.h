// mcig_launchers.h -- launch entry points of the sampling kernels, one per
// translation unit (sample_generic_*.cu, sample_fast_*.cu).
#pragma once
#include <cuda_runtime.h>
#include "mcig_common.cuh"

typedef void (*mcig_launch_fn)(const KParams &p, const FastConst *fc, int movetype, int grid, int block, size_t smem,
                               cudaStream_t st);

// general kernel: precision MCIG_PREC_*, rng RNG_PHILOX / RNG_TAPE (tape: FP64 only)
mcig_launch_fn mcig_generic_launcher(int precision, int rng);

// register-resident float kernel (mcig_fast.cuh): move MCIG_MOVE_ALL / MCIG_MOVE_VEC,
// maxd 4, 8, 16 or 32, pdf set pk (PK_ANY, or PK_GAUSS / PK_PREC / PK_MIX for a single
// sampling function of that kind); NULL otherwise
mcig_launch_fn mcig_fast_launcher(int kahan, int move, int maxd, int pk);

// step-size calibration (KMODE_CALIB) with the calibration's tail split over lanes
// (mcig_calib.cuh): all-coordinate move, one step type, no periodic domain, ndim 9..16,
// one sampling function of kind pk (PK_GAUSS or PK_PREC); NULL otherwise
mcig_launch_fn mcig_calib_launcher_pk16(int pk);

// float kernel with several lanes per chain for one mixture sampling function
// (mcig_lanes.cuh): all-coordinate move, one step type, unbound domain, maxd 32, lpc 4 or 8
// lanes per chain; NULL otherwise
mcig_launch_fn mcig_lanes_launcher(int kahan, int maxd, int lpc);

// general kernel of a plugin (include/mcig/plugin.cuh) over its user functors: launches and
// returns the launch's cudaError_t of the plugin's own CUDA runtime
typedef int (*mcig_plugin_launch_fn)(const KParams &p, int movetype, int grid, int block, size_t smem, cudaStream_t st);

// interface version of plugins against this library (with sizeof(KParams))
#define MCIG_PLUGIN_ABI 1
