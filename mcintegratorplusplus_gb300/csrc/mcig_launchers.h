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
// sampling function of that kind); moments: 1 every observable is x or x.x with float Full
// data or a Simple/Block accumulator (a kernel holding only those paths where one exists), 2
// besides that one observable per group (Full x.x, Full x, Simple/Block x.x, Simple/Block x),
// nskip 1 and ndim == maxd (a straight-line variant where one exists);
// lean: one step-size type, unbound domain and uniform (1) or Gaussian (2) draws (a kernel
// without the code of the alternatives where one exists), 0 otherwise; NULL otherwise
mcig_launch_fn mcig_fast_launcher(int kahan, int move, int maxd, int pk, int moments = 0, int lean = 0);

// step-size calibration (KMODE_CALIB) with the calibration's tail split over lanes
// (mcig_calib.cuh): all-coordinate move with uniform (gauss 0) or Gaussian (1) draws, one
// step type, no periodic domain, ndim 9..16, one sampling function of kind pk (PK_GAUSS or
// PK_PREC); NULL otherwise
mcig_launch_fn mcig_calib_launcher_pk16(int pk, int gauss);

// float kernel with several lanes per chain for one mixture sampling function
// (mcig_lanes.cuh): all-coordinate move with uniform (gauss 0) or Gaussian (1) draws, one
// step type, unbound domain, maxd 32, lpc 4 or 8 lanes per chain; NULL otherwise
mcig_launch_fn mcig_lanes_launcher(int kahan, int maxd, int lpc, int gauss);

// float kernel with two lanes per chain for one sampling function of kind pk (PK_GAUSS or
// PK_PREC) in 9..16 coordinates (mcig_pair.cuh): all-coordinate move, one step type,
// unbound domain; moments as for mcig_fast_launcher; gauss: Gaussian (1) or uniform (0) move
// draws; NULL otherwise
mcig_launch_fn mcig_pair_launcher(int kahan, int pk, int moments, int gauss);

// Metropolis-Hastings test of the learned proposal for one sampling function of kind pk
// (PK_GAUSS, PK_PREC or PK_MIX) at maxd 8, 16 or 32 (flow_accept.cu); NULL otherwise
typedef void (*mcig_flow_accept_fn)(const KParams &p, const FastConst *fc, const float *xprop, const float *lq_prop,
                                    const float *lq_cur, uint64_t cycle, int64_t krow, int64_t *nacc_flow, cudaStream_t st);
mcig_flow_accept_fn mcig_flow_accept_launcher(int maxd, int pk);
// Philox tag of the flow's accept draw (tag 3: the proposal's z in the generative pass)
enum { TAG_FLOW_ACCEPT = 4 };

// general kernel of a plugin (include/mcig/plugin.cuh) over its user functors: launches and
// returns the launch's cudaError_t of the plugin's own CUDA runtime
typedef int (*mcig_plugin_launch_fn)(const KParams &p, int movetype, int grid, int block, size_t smem, cudaStream_t st);

// interface version of plugins against this library (with sizeof(KParams))
#define MCIG_PLUGIN_ABI 1
