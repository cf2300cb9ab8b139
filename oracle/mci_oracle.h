/*
 * mci_oracle.h -- CPU oracle for the GB300 Monte Carlo integrator.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * library's hot path (MCI::integrate with its moves, sampling functions,
 * accumulators and estimators) used as the checker of the CUDA path.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 * The product (mcintegratorplusplus_gb300) never links or calls it.
 *
 * Each chain is an independent reference MCI object: same random engine
 * (std::mt19937_64 restated), same distributions (libstdc++ algorithms
 * restated), same floating-point operation order.  The oracle can record every
 * distribution output it consumes (a "tape") and can replay a tape instead of
 * the engine; the device replay mode consumes the same tape.
 *
 * Parity pinning: tests/golden/ holds outputs of the reference itself (built
 * from its sources by oracle/ref_build.sh and driven by oracle/ref_recorder.cpp)
 * and tests/test_oracle_golden.py checks this oracle against them.
 */
#ifndef MCI_ORACLE_H
#define MCI_ORACLE_H

#include <stdint.h>
#include "../include/mcig_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_mci orc_mci;

/* --- engine / distribution primitives (for known-answer tests) --- */
void orc_mt64_stream(uint64_t seed, int64_t n, uint64_t *out);
void orc_canonical_stream(uint64_t seed, int64_t n, double *out);
void orc_normal_stream(uint64_t seed, int64_t n, double *out);
void orc_uniform_int_stream(uint64_t seed, int64_t n, int64_t nvals, int64_t *out);
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* n draws of SRRDType srrd (createSymRRD's distribution with its default parameters) from a
 * fresh distribution object and std::mt19937_64(seed) */
void orc_srrd_stream(int srrd, uint64_t seed, int64_t n, double *out);

/* --- the integrator (one reference MCI per chain) --- */
orc_mci *orc_create(int ndim, int nchains);
void orc_destroy(orc_mci *h);
const char *orc_last_error(void);

int orc_set_seeds(orc_mci *h, const uint64_t *seeds); /* one seed per chain */
int orc_set_x(orc_mci *h, const double *x);           /* [nchains][ndim] */
int orc_get_x(orc_mci *h, double *x);
int orc_set_mrt2step(orc_mci *h, double step);                 /* all chains, all types */
int orc_set_mrt2step_i(orc_mci *h, int i, double step);
int orc_get_mrt2step(orc_mci *h, int chain, int i, double *step);
int orc_set_target_acceptance_rate(orc_mci *h, double rate);
int orc_set_nfind_mrt2_iterations(orc_mci *h, int n);
int orc_set_ndecorrelation_steps(orc_mci *h, int64_t n);

int orc_set_trial_move(orc_mci *h, int movetype, int srrd, int veclen, int ntypes, const int *typeEnds);
int orc_set_multistep_move(orc_mci *h, int nsteps, int sub_srrd, int sub_veclen, double sub_step);
int orc_multistep_add_pdf(orc_mci *h, int kind, const double *params, int nparams);

int orc_add_sampling_function(orc_mci *h, int kind, const double *params, int nparams);
int orc_pop_sampling_function(orc_mci *h);
int orc_clear_sampling_functions(orc_mci *h);
int orc_add_observable(orc_mci *h, int kind, const double *params, int nparams,
                       int blocksize, int nskip, int flag_equil, int estimator);
int orc_pop_observable(orc_mci *h);
int orc_clear_observables(orc_mci *h);
int orc_get_nobsdim(orc_mci *h);

int orc_set_irange(orc_mci *h, const double *lb, const double *ub); /* periodic box */
int orc_reset_domain(orc_mci *h);

int orc_set_record(orc_mci *h, int on);                   /* record tape + accept bits */
int64_t orc_get_tape(orc_mci *h, int chain, double *out, int64_t maxn); /* returns length */
int64_t orc_get_accept_bits(orc_mci *h, int chain, uint8_t *out, int64_t maxn, int64_t *main_start);
int orc_set_replay(orc_mci *h, const double *tape, int64_t stride, const int64_t *lens);
/* draws of the device kernels' Philox streams (layout 1: float kernels, 2: double kernels,
 * 0: the engine again); chain c is device chain chain0 + c at step counter ctr0[c] */
int orc_set_philox(orc_mci *h, uint64_t seed, int64_t chain0, const uint64_t *ctr0, int layout);
int orc_get_philox_counters(orc_mci *h, uint64_t *ctr);
int orc_set_chain_steps(orc_mci *h, const double *steps); /* [nchains][ntypes] */
/* log(u) - log(acceptance) of every recorded step (accepted iff <= 0) */
int64_t orc_get_margins(orc_mci *h, int chain, double *out, int64_t maxn);

/* integrate: avg/err combined over chains with the MPIMCI formula
 * (mean of averages, sqrt(sum err^2)/nchains); chain_avg/chain_err
 * (optional, [nchains][nobsdim]) receive per-chain results. */
int orc_integrate(orc_mci *h, int64_t nmc, double *avg, double *err, int do_find, int do_decorr,
                  double *chain_avg, double *chain_err, int nthreads);
double orc_get_acceptance_rate(orc_mci *h);
int orc_get_counts(orc_mci *h, int64_t *acc, int64_t *rej); /* per chain, last sample() call */
/* raw accumulator data of observable o after the last integrate: [nchains][nstore*nobs] */
int64_t orc_get_obs_data(orc_mci *h, int o, double *out, int64_t maxn);

/* --- estimators on flat [n][ndim] arrays (Estimators.cpp / MJBlocker.cpp) --- */
int orc_estimate(int estimator, int64_t n, int ndim, const double *x, double *avg, double *err);
int orc_block_estimate(int64_t n, int ndim, const double *x, int64_t nblocks, double *avg, double *err);

/* --- accumulators driven by a recorded walk (test/ut1/main.cpp:116-139) ---
 * xs[nsteps][ndim] are the walker positions after each step (wlk.xnew),
 * accepted[nsteps] the acceptance flags.  data receives nstore*nobs values. */
int64_t orc_accumulate_walk(int obs_kind, const double *params, int nparams, int ndim,
                            int blocksize, int nskip, int64_t nsteps,
                            const double *xs, const uint8_t *accepted, double *data, int64_t maxn);

#ifdef __cplusplus
}
#endif
#endif
