/*
 * mcig.h -- C ABI of the GB300-native Monte Carlo integrator (libmcigpu.so).
 *
 * The entry points mirror the reference's integrator facade mci::MCI
 * (include/mci/MCIntegrator.hpp:93-225 of DCM-UPB/MCIntegratorPlusPlus): one
 * opaque handle stands for an MCI object, except that it holds `nchains`
 * independent Markov chains that run on the GPU, one chain per thread.  With
 * nchains == 1 and MCIG_PREC_FP64 the arithmetic is the reference's.  With
 * several chains, integrate() combines the per-chain averages and errors the
 * way MPIMCI::integrate combines ranks (src/MPIMCI.cpp:85-92): mean of the
 * averages, sqrt(sum of squared errors)/nchains.
 *
 * Conventions
 *  - Every call returns an mcig_status; mcig_last_error() gives the message
 *    of the last failure in the calling thread.  Where the reference throws
 *    std::invalid_argument / std::domain_error / std::runtime_error, the
 *    matching MCIG_ERR_* code is returned and nothing is changed.
 *  - Host pointers only.  Arrays of per-chain vectors are [nchains][ndim]
 *    row-major (one reference walker per row).
 *  - All device work of a handle runs on one CUDA stream (mcig_get_stream);
 *    calls return after that work has finished.
 *  - User sampling functions and observables are device functors chosen by
 *    kind code + parameter vector (include/mcig_types.h).
 */
#ifndef MCIG_H
#define MCIG_H

#include <stddef.h>
#include <stdint.h>

#include "mcig_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mcig_mci mcig_mci;

/* last error message of the calling thread ("" if none) */
const char *mcig_last_error(void);
/* library version string */
const char *mcig_version(void);

/* MCI::MCI(int ndim) (MCIntegrator.cpp:624-649): unbound domain, uniform all-move
 * with step 0.05, target acceptance 0.5, NfindMRT2Iterations -50,
 * NdecorrelationSteps -10000, every chain at x = 0.  `device` is the CUDA
 * ordinal; `precision` an mcig_precision. */
int mcig_create(int ndim, int64_t nchains, int device, int precision, mcig_mci **out);
int mcig_destroy(mcig_mci *h);
int mcig_get_ndim(const mcig_mci *h, int *ndim);
int64_t mcig_get_nchains(const mcig_mci *h);
int mcig_set_precision(mcig_mci *h, int precision);
/* stream the handle's work is queued on (cudaStream_t as void*) */
void *mcig_get_stream(const mcig_mci *h);

/* Kernel choice: 0 automatic (register-resident float kernel where it applies,
 * else the general kernel), 1 general kernel, 2 register-resident kernel
 * (MCIG_ERR_UNSUPPORTED at integrate when the configuration needs the general one),
 * 3 multi-lane mixture kernel (mcig_set_lanes; MCIG_ERR_UNSUPPORTED where it does not apply). */
int mcig_set_kernel(mcig_mci *h, int policy);
/* Phase fusion (default off): where the register-resident kernel serves calibration, a fixed
 * burn-in and the sampling (no file output, no accept recording), integrate runs the three
 * phases of every chain in one launch, so chains whose step calibration converges early
 * sample while the others still calibrate.  Results are those of separate launches; the
 * timings then report the whole launch as sampling time.  Off by default: when a few chains
 * calibrate for many iterations, their calibration competes with the other chains' sampling
 * for instruction issue and then their own sampling ends the launch late (65,536 chains of a
 * 16-D correlated Gaussian: 66.3 ms fused against 58.5 ms for the three launches). */
int mcig_set_phase_fusion(mcig_mci *h, int on);
/* Split calibration tail (default on): where the register-resident kernel calibrates an
 * all-coordinate move with one step-size type, no periodic domain, ndim 9..16 and one exp(-x.x)
 * or precision-matrix sampling function, the chains still calibrating when at most 8 of
 * their warp's 32 remain continue on 4 lanes each (4 coordinates per lane, the proposal
 * exchanged by warp shuffles).  Step sizes, walkers and counts are identical to the one-lane
 * calibration; only the time changes.  0 turns it off.  No counterpart in the reference,
 * whose MCI::findMRT2Step (src/MCIntegrator.cpp:87-168) calibrates one chain. */
int mcig_set_calibration_split(mcig_mci *h, int on);

/* Multi-lane kernels.  lpc = 0 (default): automatic, i.e. two lanes per chain for the
 * configurations of lpc = 2 with at most 32,768 chains unless every observable is x or x.x
 * (whose one-lane variant is as fast), else one; lpc = 1: one lane per chain.
 * lpc = 2: a float handle with one exp(-x.x) or precision-matrix sampling function in 9..16
 * coordinates (all-coordinate uniform or Gaussian move, one step type, unbound domain,
 * observables without exp() or coordinate blocks) runs burn-in and sampling (and the
 * calibration when its split tail is off) with 2 lanes per chain: lane group l draws and
 * moves coordinates [8l, 8l+8), the proposal is gathered with warp shuffles and each lane
 * forms 8 rows of U x (mcig_pair.cuh).  Results are bit-identical to the one-lane kernel;
 * the point is latency hiding where one lane per chain leaves few warps per SM (16,384
 * chains: 3.4 warps per SM with one lane at 124 registers, 6.7 with two at 80 registers;
 * measured sampling launch 18.9 against 23.9 ms; at 65,536 chains the one-lane kernel is
 * faster, 35.8 against 41.5 ms).
 * lpc = 4 or 8: a float handle whose single
 * sampling function is a mixture of at most 8 Gaussians (17..32 coordinates, all-coordinate
 * uniform or Gaussian move, one step type, unbound domain) runs its calibration, burn-in and
 * sampling with lpc lanes per chain: lane group l draws and moves coordinates [l*ndim/lpc,
 * ...), the proposal is gathered with warp shuffles and each lane evaluates its mixture
 * components.  Results are bit-identical to the one-lane kernel; the point is occupancy
 * (16,384 chains fill 3.4 warps of an SM with one lane per chain, 27 with 8).  No
 * counterpart in the reference, whose MCI runs one chain on one thread. */
int mcig_set_lanes(mcig_mci *h, int lpc);
/* Metropolis decision certified in double (the precision form; multi-lane kernel only, else
 * MCIG_ERR_UNSUPPORTED at integrate).  mode 1: the float log-space test decides unless its
 * margin |log u - (log p(x') - log p(x))| is below (2^-12 + 2^-18 (|log p(x)| + |log p(x')|)),
 * where the log densities of the float positions are recomputed in double and the double test
 * log u <= log p(x') - log p(x) decides (MCI::doStepMRT2, MCIntegrator.cpp:343, in log space).
 * mode 2 (diagnostic) takes the double test on every step.  mcig_get_decision_stats gives,
 * for the last integrate, the steps tested in double, how many float decisions the double
 * test reversed, and the largest float margin among the reversed ones. */
int mcig_set_fp64_decision(mcig_mci *h, int mode);
int mcig_get_decision_stats(const mcig_mci *h, int64_t *checked, int64_t *reversed, double *max_margin);

/* Chunked sampling (default 1: off): where the register-resident one-lane kernel
 * samples, no observable uses a SimpleAccumulator and float FullAccumulator samples take the
 * Uncorrelated estimator, the main sampling runs as n launches of equal length (a multiple of
 * every block length), and the estimator of each finished chunk's Full rows runs on a
 * low-priority stream beside the next launch.  Results are identical to one launch and the
 * one-pass estimator; the estimation's pass over the Full samples can overlap the sampling
 * where the sampling leaves the SMs room (with 65,536 chains of the 16-D workload it does not:
 * measured slower, hence off).  No counterpart in the reference, whose MCI::sample
 * (MCIntegrator.cpp:290-321) is one loop. */
int mcig_set_sampling_chunks(mcig_mci *h, int n);

/* MCI::setSeed (MCIntegrator.cpp:547-550).  Philox4x32-10 key; chain c draws
 * from counter (step, c).  */
int mcig_set_seed(mcig_mci *h, uint64_t seed);

/* MCI::setX (:594-604): x is [nchains][ndim], or [ndim] broadcast when n == 1 */
int mcig_set_x(mcig_mci *h, const double *x, int64_t n);
int mcig_get_x(mcig_mci *h, double *x /* [nchains][ndim] */);
/* MCI::centerX (MCIntegrator.hpp:105): domain centre (0 in the unbound domain) */
int mcig_center_x(mcig_mci *h);

/* MCI::setMRT2Step (:557-579) for every chain; getMRT2Step (:581-585) of chain 0
 * (0 for a non-existing index, as the reference) */
int mcig_set_mrt2step(mcig_mci *h, double step);
int mcig_set_mrt2step_i(mcig_mci *h, int i, double step);
int mcig_get_mrt2step(const mcig_mci *h, int64_t chain, int i, double *step);
int mcig_get_nstepsizes(const mcig_mci *h, int *n);
/* per-chain step sizes, [nchains][nstepsizes] */
int mcig_get_mrt2steps(const mcig_mci *h, double *steps);

/* MCI::setTargetAcceptanceRate / setNfindMRT2Iterations / setNdecorrelationSteps
 * (MCIntegrator.hpp:113-123): N < 0 automatic with at most |N|, 0 off, N > 0 fixed */
int mcig_set_target_acceptance_rate(mcig_mci *h, double rate);
int mcig_set_nfind_mrt2_iterations(mcig_mci *h, int n);
int mcig_set_ndecorrelation_steps(mcig_mci *h, int64_t n);

/* MCI::setTrialMove(SRRDType, veclen, ntypes, typeEnds) (MCIntegrator.cpp:431-446)
 * and setTrialMove(MoveType) (:423-429).  movetype MCIG_MOVE_ALL ignores
 * veclen; MCIG_MOVE_VEC uses veclen >= 1; MCIG_MOVE_MULTISTEP installs the
 * default MultiStepMove(ndim) (MultiStepMove.hpp:49-52).  Every SRRDType runs on the
 * device: in replay mode from the reference's recorded draws (bit for bit), with Philox draws
 * as the transforms of mcig_common.cuh move_draws_srrd. */
int mcig_set_trial_move(mcig_mci *h, int movetype, int srrd, int veclen, int ntypes, const int *typeEnds);
/* MultiStepMove(ndim, nsteps) with sub-move SRRDVecMove(ndim/veclen, veclen, step)
 * (MultiStepMove.hpp:40-52, src/MultiStepMove.cpp:6-75) */
int mcig_set_multistep_move(mcig_mci *h, int nsteps, int sub_srrd, int sub_veclen, double sub_step);
/* MultiStepMove::addSamplingFunction (src/MultiStepMove.cpp:61-67) */
int mcig_multistep_add_pdf(mcig_mci *h, int kind, const double *params, int nparams);

/* MCI::addSamplingFunction / popSamplingFunction / clearSamplingFunctions (MCIntegrator.hpp:181-184) */
int mcig_add_sampling_function(mcig_mci *h, int kind, const double *params, int nparams);
int mcig_pop_sampling_function(mcig_mci *h);
int mcig_clear_sampling_functions(mcig_mci *h);
int mcig_get_npdf(const mcig_mci *h, int *n);

/* MCI::addObservable(obs, blocksize, nskip, flag_equil, EstimatorType) (MCIntegrator.cpp:451-465);
 * blocksize 0 -> SimpleAccumulator, 1 -> FullAccumulator, >1 -> BlockAccumulator
 * (Factories.hpp:24-38).  mcig_add_observable_default applies the defaults of
 * addObservable(obs, blocksize, nskip) (MCIntegrator.hpp:161-164). */
int mcig_add_observable(mcig_mci *h, int kind, const double *params, int nparams, int blocksize, int nskip,
                        int flag_equil, int estimator);
int mcig_add_observable_default(mcig_mci *h, int kind, const double *params, int nparams, int blocksize, int nskip);
int mcig_pop_observable(mcig_mci *h);
int mcig_clear_observables(mcig_mci *h);
int mcig_get_nobs(const mcig_mci *h, int *n);
int mcig_get_nobsdim(const mcig_mci *h, int *n);
/* FullAccumulator samples stored as float (32) or double (64, default) */
int mcig_set_full_storage(mcig_mci *h, int bits);

/* MCI::setIRange (:398-408): orthorhombic periodic box; resetDomain (:390-396) */
int mcig_set_irange(mcig_mci *h, const double *lbounds, const double *ubounds);
int mcig_reset_domain(mcig_mci *h);

/* MCI::integrate (MCIntegrator.cpp:43-82).  average/error have getNObsDim()
 * entries (combined over chains).  chain_avg / chain_err, if not NULL, receive
 * [nchains][nobsdim] per-chain results. */
int mcig_integrate(mcig_mci *h, int64_t nmc, double *average, double *error, int do_find_mrt2step,
                   int do_decorrelation);
int mcig_get_chain_results(const mcig_mci *h, double *chain_avg, double *chain_err);
/* MCI::storeObservablesOnFile / storeWalkerPositionsOnFile / clear*File
 * (src/MCIntegrator.cpp:495-542): during the main sampling of the next integrate
 * calls, every freq-th step of chain 0 is written as the reference writes it
 * ("<step> v1 v2 ... " and "<step>   x1   x2 ..."), observables as the values of
 * each accumulator's last accumulation.  The general kernel runs while a file is set. */
int mcig_store_observables_on_file(mcig_mci *h, const char *path, int freq);
int mcig_clear_observable_file(mcig_mci *h);
int mcig_store_walker_positions_on_file(mcig_mci *h, const char *path, int freq);
int mcig_clear_walker_file(mcig_mci *h);
/* MCI::getAcceptanceRate (:587-592) of the last sampling run, over all chains */
int mcig_get_acceptance_rate(const mcig_mci *h, double *rate);
/* per-chain accepted / rejected counts of the last sampling run */
int mcig_get_counts(const mcig_mci *h, int64_t *acc, int64_t *rej);

/* Accumulator data of observable o after the last integrate, in the
 * reference's per-chain layout [nchains][nstore][nobs] (AccumulatorInterface::getData,
 * AccumulatorInterface.hpp:81).  n receives the element count when data is NULL. */
int mcig_get_obs_data(const mcig_mci *h, int o, double *data, int64_t *n);

/* The same data for the chains [c0, c0 + nc) only, [nc][nstore][nobs] (n receives the
 * element count): a few chains' FullAccumulator series without copying every chain's. */
int mcig_get_obs_data_chains(const mcig_mci *h, int o, int64_t c0, int64_t nc, double *data, int64_t *n);
/* Philox step counter of every chain ([nchains]): the steps (calibration, burn-in and
 * sampling) the chain has drawn since mcig_set_seed.  Step t of chain c draws from Philox
 * counter (t lo, t hi, c, substep << 16 | tag << 12 | block) with key (seed lo, seed hi).
 * No counterpart in the reference, whose chains share one sequential engine. */
int mcig_get_step_counters(const mcig_mci *h, uint64_t *ctr);

/* Replay mode (tests): consume recorded distribution outputs instead of
 * Philox draws.  tape is [nchains][stride] in the order the reference draws
 * them; lens the per-chain lengths.  Requires MCIG_PREC_FP64.  NULL switches
 * back to Philox. */
int mcig_set_replay(mcig_mci *h, const double *tape, int64_t stride, const int64_t *lens);
/* record the accept/reject decision of every main-sampling step into a
 * [nsteps][nchains] byte array readable with mcig_get_accept_bits */
int mcig_set_record_accepts(mcig_mci *h, int on);
int mcig_get_accept_bits(const mcig_mci *h, uint8_t *bits, int64_t *nsteps);

/* Estimators on host arrays x[n][ndim] computed on the device
 * (src/Estimators.cpp:36-293, src/MJBlocker.cpp:19-154).  `estimator` is an
 * mcig_estimator.  MCIG_PREC_FP64 arithmetic, reference operation order. */
int mcig_estimate(int device, int estimator, int64_t n, int ndim, const double *x, double *average, double *error);

/* Accumulator of one observable driven by a recorded walk (test/ut1 pattern):
 * xs[nsteps][ndim] walker positions after each step, accepted[nsteps] flags.
 * data receives nstore*nobs values (AccumulatorInterface.cpp:31-122). */
int mcig_accumulate_walk(int device, int obs_kind, const double *params, int nparams, int ndim, int blocksize,
                         int nskip, int64_t nsteps, const double *xs, const uint8_t *accepted, double *data,
                         int64_t *ndata);

/* Device-side timing of the last integrate (milliseconds per phase:
 * calibration, burn-in, sampling, estimation) and the number of kernels it launched. */
int mcig_get_last_timings(const mcig_mci *h, double *ms4, int64_t *nlaunches);

/* ------------------------------------------------------------------------
 * Learned proposal (no counterpart in the reference's code; the reference's
 * MCI API is extended by one call).  An affine-coupling normalizing flow
 * (RealNVP: L coupling layers, MLP hidden width 128, bf16 tensor-core GEMMs
 * with float accumulation, float master weights trained with Adam by
 * maximum likelihood on chain states) is used as an independence
 * Metropolis-Hastings proposal mixed with the local moves, so the target is
 * unchanged.  Flow definition and parameter layout: oracle/flow_oracle.py.
 * ------------------------------------------------------------------------ */
typedef struct mcig_flow mcig_flow;
int64_t mcig_flow_nparams(int ndim, int nlayers);
/* ndim even, <= 32; nlayers <= 16; hidden must be 128 */
int mcig_flow_create(int ndim, int nlayers, int hidden, uint64_t seed, int device, mcig_flow **out);
int mcig_flow_destroy(mcig_flow *f);
int mcig_flow_get_params(const mcig_flow *f, float *theta, int64_t *n);
int mcig_flow_set_params(mcig_flow *f, const float *theta, int64_t n);
/* Self-test of the flow's 5th-generation tensor-core path (tcgen05.mma from shared-memory
 * descriptors, accumulator in tensor memory): d[128][n] = a[128][k] b[n][k]^T with bf16
 * inputs (raw 16-bit patterns) and f32 accumulation, one CTA.  n, k multiples of 16 in
 * [16, 256].  MCIG_ERR_TIMEOUT when the MMA's completion was not seen within the bounded wait. */
int mcig_flow_tc_selftest(int device, const uint16_t *a, const uint16_t *b, int n, int k, float *d);
/* the kernel of the flow's passes (proposals, densities, training's density pass): 0 (default)
 * register-fused mma.sync (one warp carries 16 rows through every layer with the hidden
 * activations in registers; two row sets per launch for the learned proposal's densities),
 * 1 tcgen05 with TMEM accumulators, 2 mma.sync with the hidden activations in shared memory.
 * 0 and 2 give the same numbers bit for bit; all three agree with the oracle at bf16 tolerance */
int mcig_flow_set_tensor_path(mcig_flow *f, int tc);
/* generative direction: x = f(z) and log q(x) for z[n][ndim] (host arrays) */
int mcig_flow_forward(mcig_flow *f, const double *z, int64_t n, double *x, double *logq);
/* density direction: z = f^-1(x) and log q(x) */
int mcig_flow_inverse(mcig_flow *f, const double *x, int64_t n, double *z, double *logq);
/* loss -mean log q(x) and its gradient (nparams floats) */
int mcig_flow_loss_grad(mcig_flow *f, const double *x, int64_t n, double *loss, float *grad);
/* `steps` Adam steps on minibatches of `batch` rows drawn from x[n][ndim] */
int mcig_flow_train(mcig_flow *f, const double *x, int64_t n, int steps, int batch, double lr, double *last_loss);
/* MCI::integrate with the learned proposal.  Calibration and burn-in with the
 * local move; then `train_steps` adaptation cycles, each of period - 1 local
 * steps, a snapshot of the chain positions and one Adam step (learning rate
 * lr) on `batch` rows drawn from that snapshot, with flow proposals from the
 * first quarter of the cycles on; then nmc recorded steps, every `period`-th
 * one a flow proposal (period 5 = 1:4 with the local move).  refresh > 0
 * adds one Adam step every `refresh` steps while sampling; 0 freezes the
 * flow.  Every observable must use a FullAccumulator (blocksize 1) with
 * nskip 1.  flow_acceptance receives the acceptance rate of the recorded
 * flow proposals. */
int mcig_integrate_flow(mcig_mci *h, mcig_flow *f, int64_t nmc, int period, int64_t refresh, int train_steps, int batch,
                        double lr, double *average, double *error, int do_find_mrt2step, int do_decorrelation,
                        double *flow_acceptance);

/* ------------------------------------------------------------------------
 * Batched integration: many independent MCI::integrate calls (one handle each,
 * any ndim <= 64, its own sampling functions, move, observables and seed) run
 * by ONE persistent kernel launch whose warps pull work items (up to 32 chains of
 * one integral) longest-first from one atomic queue over the whole batch; the
 * launch, the estimators and the read-back are one CUDA graph.  Integrals of the
 * block-separable form (single-coordinate MultiStepMove, isotropic Gaussian
 * factors over coordinate ranges as sampling functions and sub-pdfs, x.x per
 * factor or in all) run a sampler that keeps the walker in shared memory and the
 * log densities as per-range sums of squares; every other integral runs the
 * general sampler in the same launch.  All handles use one precision and draw
 * source: MCIG_PREC_FP32 / FP32_ACC64 with Philox, or MCIG_PREC_FP64 with Philox
 * or replayed draws (the general double sampler: each chain's numbers are those of
 * its own integrate).  Handles need a sampling function, burn-in N >= 0 and
 * observables with the Uncorrelated (Block/Full, double data) or Noop estimator.
 * ------------------------------------------------------------------------ */
typedef struct mcig_batch mcig_batch;
int mcig_batch_create(mcig_mci **handles, int n, const int64_t *nmc, int do_find_mrt2step, int do_decorrelation,
                      mcig_batch **out);
/* one run of every integral; avg/err receive each handle's getNObsDim() values in handle order */
int mcig_batch_run(mcig_batch *b, double *avg, double *err);
int mcig_batch_destroy(mcig_batch *b);
/* device time of the last run (graph launch to completion), milliseconds */
int mcig_batch_last_ms(const mcig_batch *b, double *ms);
/* threads per block of the launch and, per ndim bucket (1-8, 9-16, 17-32, 33-64), the
 * unroll (1, 2, 4) of the block-separable sampler's sub-step loop */
int mcig_batch_get_tuning(const mcig_batch *b, int *block, int *unroll /* [4] */);
int mcig_batch_set_tuning(mcig_batch *b, int block, const int *unroll /* [4], NULL: unchanged */);
/* time 64/128/256 threads per block, then per bucket the three unrolls, keep the fastest;
 * cache file optional (keyed by the batch's shape) */
int mcig_batch_autotune(mcig_batch *b, const char *cache_path);

/* ------------------------------------------------------------------------
 * Plugins: user sampling functions and observables compiled for the device
 * (include/mcig/plugin.cuh).  They replace the reference's user classes derived
 * from SamplingFunctionInterface / ObservableFunctionInterface, passed to
 * MCI::addSamplingFunction (MCIntegrator.hpp:174-184) and MCI::addObservable
 * (:152-172).  A plugin is a shared library built with MCIG_PLUGIN; after
 * mcig_set_plugin the kinds MCIG_PDF_USER + k and MCIG_OBS_USER + k name its k-th
 * sampling function and observable (addSamplingFunction / addObservable /
 * mcig_multistep_add_pdf, parameters handed to the functor).  Handles with plugin
 * kinds run the plugin's general kernel in every precision; the register-resident
 * kernel, batches, the learned proposal, observable file output and the LOGPDF
 * observable are for built-in kinds.  A plugin stays loaded while handles use it.
 * ------------------------------------------------------------------------ */
typedef struct mcig_plugin mcig_plugin;
/* dlopen the library; MCIG_ERR_INVALID_ARGUMENT when it is not a plugin of this version */
int mcig_plugin_load(const char *path, mcig_plugin **out);
int mcig_plugin_unload(mcig_plugin *pl);
/* number of sampling functions and observables of the plugin */
int mcig_plugin_counts(const mcig_plugin *pl, int *npdf, int *nobs);
/* attach (or, with NULL, detach) the plugin whose kinds the handle may use */
int mcig_set_plugin(mcig_mci *h, const mcig_plugin *pl);
/* number of trial moves of the plugin (MCIG_PLUGIN_MOVES; 0 for MCIG_PLUGIN) */
int mcig_plugin_nmoves(const mcig_plugin *pl, int *nmove);
/* the plugin's k-th trial move as the handle's move: MCI::setTrialMove(unique_ptr<
 * TrialMoveInterface>) (MCIntegrator.hpp:140, MCIntegrator.cpp:423-432).  params are
 * handed to the move (UserArgs); its step sizes (at most MCIG_MAXTYPES = 4, set to the move's
 * step0 values in every chain) are calibrated by findMRT2Step like the built-in moves' and
 * read with mcig_get_mrt2step; a move without step sizes skips the calibration.  The move
 * runs in the plugin's general kernel, at the top level (not as a MultiStepMove sub-move).
 * Errors: no plugin, k out of range, nproto above the move's max_nproto, more than
 * MCIG_MAXTYPES step sizes, a step size index out of range. */
int mcig_set_user_move(mcig_mci *h, int k, const double *params, int nparams);

/* Philox4x32-10 block (for known-answer tests of the device generator) */
int mcig_philox_block(int device, const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* MJBlocker estimate of device data that allocates no device memory.  No
 * counterpart in the reference: it serves callers that cannot call cudaMalloc
 * (device memory owned by their own pool, allocation forbidden after start-up,
 * or a loop that must not synchronize the device).  d_x[n][ndim], d_avg[ndim]
 * and d_err[ndim] are device pointers; the work is queued on `stream`
 * (cudaStream_t, NULL for the default stream) and the call returns without
 * waiting.  Scratch is a file-scope device array of MCIG_NOALLOC_MAX_VALUES
 * doubles (16 MiB on every device that loads the library, until exit):
 * n*ndim above that is rejected with MCIG_ERR_INVALID_ARGUMENT, as is an n
 * that is not a power of two.  The first call on a device looks up the
 * array's device address (make that call before any stream capture).  All
 * calls share the array, so calls that overlap on the GPU race: order them. */
#define MCIG_NOALLOC_MAX_VALUES (1 << 21)
#define MCIG_NOALLOC_MAX_DEVICES 64
int mcig_mjblocker_estimate_noalloc(const double *d_x, int64_t n, int ndim, double *d_avg, double *d_err,
                                    void *stream);

#ifdef __cplusplus
}
#endif
#endif
