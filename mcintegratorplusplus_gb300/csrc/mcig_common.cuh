// mcig_common.cuh -- parameter block, Philox generator and draw helpers shared by the
// sampling kernels (mcig_generic.cuh, mcig_fast.cuh); one chain per thread.
//
// A launch runs `nsteps` steps of MCI::sample (reference src/MCIntegrator.cpp:273-321)
// for every chain: trial move (SRRDAllMove.hpp:67-80, SRRDVecMove.hpp:75-96,
// src/MultiStepMove.cpp:6-47), domain (OrthoPeriodicDomain.cpp:38-61), product of
// sampling-function acceptances (SamplingFunctionContainer.cpp:41-48), the
// Metropolis test (MCIntegrator.cpp:343) and the accumulators
// (AccumulatorInterface.cpp:31-114, Simple/Block/FullAccumulator.cpp), or the
// step-size calibration loop of MCI::findMRT2Step (MCIntegrator.cpp:87-168).
//
// Memory layout (chain-minor so that a warp's accesses are coalesced):
//   x[ndim][nchains], step[ntypes][nchains], Full data [nstore][nobs][nchains],
//   Block data [nblocks][nobs][nchains], Simple data [nobs][nchains].
//
// Random numbers: Philox4x32-10 keyed by the seed; the block for draw group
// (substep, tag, b) of step t of chain c has counter (t lo, t hi, c,
// substep<<16 | tag<<12 | b), so every draw is addressable and a chain's stream
// does not depend on the launch configuration.  Replay mode reads the
// reference's recorded distribution outputs ("tape") in its draw order.
#pragma once

#include <cstdint>
#include <map>
#include <mutex>
#include <type_traits>
#include <utility>
#include <cuda_runtime.h>

#include "../../include/mcig_types.h"

#define MCIG_MAXPDF 4
#define MCIG_MAXOBS 8
#define MCIG_MAXTYPES 4
#define MCIG_PERIODIC_MAXWRAP 64
#define MCIG_MAXDIM 64
#define MCIG_FAST_BLOCK 64 // threads per block of the register-resident kernel (slot stride)
#define MCIG_FCONST 2080 // floats of sampling-function data in the parameter block (register-resident kernel)

// Shared-memory attributes of kernel k on the current device, set through the runtime once
// per kernel and device (they persist for the process): the carveout at its maximum, and the
// dynamic shared-memory limit raised whenever a launch asks for more than any before it.
// Loops of short launches (the learned proposal's local steps) would otherwise spend host
// time on attribute calls at every launch.
inline void mcig_smem_attrs(const void *k, size_t smem)
{
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, size_t> limit; // (kernel, device) -> dynamic limit set
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> g(mu);
    auto it = limit.find(std::make_pair(k, dev));
    if (it == limit.end()) {
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
        it = limit.emplace(std::make_pair(k, dev), (size_t)48 * 1024).first;
    }
    if (smem > it->second) {
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        it->second = smem;
    }
}

enum { RNG_PHILOX = 0, RNG_TAPE = 1 };
// KMODE_FUSED (register-resident kernel): calibration (MIN_STAT fuse_calib, none if 0), burn-in
// (fuse_burnin steps) and sampling (nsteps) of each chain in one launch
enum { KMODE_STEPS = 0, KMODE_SAMPLE = 1, KMODE_CALIB = 2, KMODE_FUSED = 3 };

struct PdfDesc {
    int kind;
    int poff;     // offset of the parameters in KParams::params (double) / the float blob
    int np;
    int b0, b1;   // GAUSS_BLOCK bounds
    double c;     // GAUSS_BLOCK: 1/(2 w^2)
    int foff;     // float path: offset of this pdf's data in the shared-memory blob
    int fstride;  // float path: coordinate stride of that data (>= ndim, zero-padded)
    int nproto;   // plugin kinds: proto values of this sampling function
};

struct ObsDesc {
    int kind;
    int nv;       // number of values
    int poff, np; // parameters (double) in KParams::params
    int acc;      // mcig_accumulator
    int nskip;
    int bs;       // block size (Block)
    int voff;     // offset of this observable's values in the accumulator arrays
    void *data;   // device data (see layout above)
    int64_t nstore;
    int full32;   // Full data stored as float
    // n / d == __umulhi(n, magic) >> shift for n < 2^31 (register-resident kernel)
    uint32_t bs_magic, bs_shift, sk_magic, sk_shift;
    double inv_bs; // 1. / bs (Block normalisation, BlockAccumulator.cpp)
    int lslot;     // multi-lane kernel (mcig_lanes.cuh): first accumulator slot of a lane
};

struct KParams {
    int ndim;
    int nchains;
    int64_t nsteps;     // steps of this launch (KMODE_STEPS / KMODE_SAMPLE / KMODE_FUSED), MIN_STAT (KMODE_CALIB)
    int mode;
    int64_t fuse_calib, fuse_burnin; // KMODE_FUSED: MIN_STAT of the calibration (0: none), burn-in steps
    // trial move
    int srrd, veclen, ntypes;
    int typeEnds[MCIG_MAXTYPES];
    int ms_nsteps, ms_srrd, ms_veclen, ms_npdf;
    PdfDesc ms_pdf[MCIG_MAXPDF];
    // user trial move (MCIG_MOVE_USER): index in the plugin's move list, its parameters at
    // params[umove_poff .. + umove_np), its proto values, and the upper limit of each step
    // size at params[step_lim_off + t] (the smallest 0.5 * domain size over the coordinates
    // that step size t moves)
    int umove, umove_poff, umove_np, umove_nproto, step_lim_off;
    // sampling functions
    int npdf;
    PdfDesc pdf[MCIG_MAXPDF];
    const double *params;   // all pdf / observable parameters (double)
    const float *fblob;     // float path: pdf data copied into shared memory
    int fblob_len;          // floats
    // observables
    int nobs;
    int nobsdim;
    ObsDesc obs[MCIG_MAXOBS];
    // domain
    int periodic;
    const double *lb, *ub;
    // chain state
    double *x;
    double *step;
    uint64_t *ctr;          // Philox step counter per chain
    int64_t *tpos;          // tape cursor per chain
    int64_t *nacc, *nrej;   // counts of this launch (KMODE_CALIB: of the last iteration)
    uint8_t *bits;          // optional [nsteps][nchains] accept record
    int64_t acc_offset;     // Full accumulators: row of this launch's first accumulation
    int64_t r0;             // register-resident kernel, chunked sampling: step index of this launch's
                            // first step in the whole sampling run (accumulation and block indices)
    int acc_counts;         // 1: add this launch's counts to nacc/nrej (later chunks of a run)
    const uint8_t *active;  // optional: chains with active[c] == 0 skip this launch
    // file output (storeObservablesOnFile / storeWalkerPositionsOnFile): chain 0 records
    // its walker after the steps dump_steps[0..ndump) (ascending) into dump_x[ndump][ndim]
    const int64_t *dump_steps;
    int64_t ndump;
    double *dump_x;
    // random numbers
    uint32_t key0, key1;
    const double *tape;
    int64_t tape_stride;
    const int64_t *tape_len;
    // calibration (MCI::findMRT2Step)
    int nfind;
    double target;
    double step_max;        // 0.5 * domain size (same for every index in the unbound domain)
    const double *step_max_i; // periodic: 0.5*(ub-lb) per index
    // error reporting
    int *status;
    // multi-lane mixture kernel (mcig_lanes.cuh): Metropolis decision certified in double near
    // the float threshold (1), or on every step (2, diagnostic), with counters [checked,
    // reversed, largest float margin of a reversed decision as float bits] (NULL: none)
    int f64_decide;
    unsigned long long *dstats;
    // register-resident kernel, x / x.x variant: the observables ordered as four groups (Full
    // x.x, Full x, Simple/Block x.x, Simple/Block x) with these counts (set by its launcher)
    int mgroup[4];
    int mgroup_slots;   // at most one observable per group, group g's at obs[g]
};

// Register-resident kernel only: Philox round keys (key + r*W for r = 0..9), the
// one-hot step-type table of the coordinates, and the sampling-function data at fixed offsets (Cholesky factor U[MAXD][MAXD] at
// 0, mixture [nc, per component: log-normalisation, m[MAXD], 1/s[MAXD]] at
// MAXD*MAXD), passed as a second kernel parameter so that the unrolled loops
// read them as constant-bank operands.
struct FastConst {
    uint32_t rk[20];
    float tw[MCIG_MAXTYPES][32]; // tw[t][i] = 1 if coordinate i < ndim has step type t, else 0
    float fconst[MCIG_FCONST];
};

// ------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)
// ------------------------------------------------------------------------
struct P4 { uint32_t a, b, c, d; };

__device__ __forceinline__ P4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                            uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) { // each 32x32 -> 64-bit product is one wide multiply
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c0 = n0; c1 = (uint32_t)p1; c2 = n2; c3 = (uint32_t)p0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return P4{c0, c1, c2, c3};
}

// Counter layout of one draw block: (step lo, step hi, chain, sub), with
// sub = (substep << 16) | (tag << 12) | block.  substep is 0 for the outer
// move and 1 + s for sub-step s of a MultiStepMove.
enum { TAG_MOVE = 0, TAG_ACCEPT = 1, TAG_INDEX = 2 };

// the same generator with the round keys precomputed (rk[2r], rk[2r+1] = key + r*W)
__device__ __forceinline__ P4 philox4x32_10_rk(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, const uint32_t *rk)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ rk[2 * r];
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ rk[2 * r + 1];
        c0 = n0; c1 = (uint32_t)p1; c2 = n2; c3 = (uint32_t)p0;
    }
    return P4{c0, c1, c2, c3};
}

struct PhiloxCtx {
    uint32_t k0, k1, s0, s1, chain;
    __device__ __forceinline__ P4 block(uint32_t substep, uint32_t tag, uint32_t b) const
    {
        return philox4x32_10(s0, s1, chain, (substep << 16) | (tag << 12) | b, k0, k1);
    }
};

__device__ __forceinline__ float u01_f(uint32_t w) { return (float)(w >> 8) * 5.9604644775390625e-08f; }           // [0,1)
__device__ __forceinline__ float u01_open0_f(uint32_t w) { return (float)((w >> 8) + 1u) * 5.9604644775390625e-08f; } // (0,1]
__device__ __forceinline__ double u01_d(uint32_t hi, uint32_t lo)
{
    return (double)(((uint64_t)hi << 21) | (uint64_t)(lo >> 11)) * 1.1102230246251565e-16; // [0,1), 53 bits
}

// two standard normals from two uniforms (Box-Muller)
__device__ __forceinline__ void box_muller_f(uint32_t w0, uint32_t w1, float &z0, float &z1)
{
    const float u = ((float)(w0 >> 8) + 0.5f) * 5.9604644775390625e-08f; // (0,1), never 0 or 1
    const float t = -1.38629436f * __log2f(u);                            // -2 ln u > 0
    const float r = t * rsqrtf(t);
    float s, c;
    __sincosf(6.28318530717958648f * (u01_f(w1) - 0.5f), &s, &c);
    z0 = r * c;
    z1 = r * s;
}

__device__ __forceinline__ void box_muller_d(P4 q, double &z0, double &z1)
{
    const double u = 1.0 - u01_d(q.a, q.b); // (0,1]
    const double r = sqrt(-2.0 * log(u));
    double s, c;
    sincospi(2.0 * u01_d(q.c, q.d), &s, &c);
    z0 = r * c;
    z1 = r * s;
}

// Move draws for coordinates [b*CPB, b*CPB+CPB) from one Philox block.
// float: 4 coordinates per block (4 uniforms or 2 Box-Muller pairs).
// double: 2 coordinates per block (2 uniforms of 53 bits or 1 pair).
template <class R> struct Cpb { static constexpr int v = 4; };
template <> struct Cpb<double> { static constexpr int v = 2; };

template <class R>
__device__ __forceinline__ void move_draws(P4 q, int gaussian, R *d /* Cpb<R>::v */);

template <>
__device__ __forceinline__ void move_draws<float>(P4 q, int gaussian, float *d)
{
    if (gaussian) {
        box_muller_f(q.a, q.b, d[0], d[1]);
        box_muller_f(q.c, q.d, d[2], d[3]);
    } else {
        d[0] = u01_f(q.a) * 2.0f - 1.0f;
        d[1] = u01_f(q.b) * 2.0f - 1.0f;
        d[2] = u01_f(q.c) * 2.0f - 1.0f;
        d[3] = u01_f(q.d) * 2.0f - 1.0f;
    }
}

template <>
__device__ __forceinline__ void move_draws<double>(P4 q, int gaussian, double *d)
{
    if (gaussian) {
        box_muller_d(q, d[0], d[1]);
    } else {
        d[0] = u01_d(q.a, q.b) * 2.0 - 1.0;
        d[1] = u01_d(q.c, q.d) * 2.0 - 1.0;
    }
}

// Move draws of every SRRDType with the standard library's default parameters
// (createSymRRD specialisations, TrialMoveInterface.hpp:113-200, and the
// SymmetrizedPRRD wrapper :82-98, which flips the sign with probability 1/2):
//   Student t (n = 1) and Cauchy(0, 1):  tan(pi (u - 1/2))
//   Fisher F(1, 1) = (z1/z2)^2 = Cauchy^2,  symmetrized
//   Exponential(1) = Gamma(1, 1) = Weibull(1, 1):  -log u,  symmetrized
//   Lognormal(0, 1): exp(z),  Chi-squared(1): z^2 (z standard normal),  symmetrized
// Uniform and Gaussian are move_draws().  float: 4 values per Philox block, double: 2;
// a symmetrized value takes its sign from a bit of the block that its magnitude leaves
// unused (the low bits below the 24 / 53 bits of the uniforms).
template <class R>
__device__ __forceinline__ void move_draws_srrd(P4 q, int srrd, R *d /* Cpb<R>::v */);

__device__ __forceinline__ float signed_by(uint32_t w, int bit, float v) { return ((w >> bit) & 1u) ? -v : v; }
__device__ __forceinline__ double signed_by(uint32_t w, int bit, double v) { return ((w >> bit) & 1u) ? -v : v; }

template <>
__device__ __forceinline__ void move_draws_srrd<float>(P4 q, int srrd, float *d)
{
    const uint32_t w[4] = {q.a, q.b, q.c, q.d};
    switch (srrd) {
    case MCIG_SRRD_UNIFORM: move_draws<float>(q, 0, d); return;
    case MCIG_SRRD_GAUSSIAN: move_draws<float>(q, 1, d); return;
    case MCIG_SRRD_STUDENT:
    case MCIG_SRRD_CAUCHY:
    case MCIG_SRRD_FISHER:
        for (int k = 0; k < 4; ++k) {
            float sn, cs;
            sincospif(((float)(w[k] >> 8) + 0.5f) * 5.9604644775390625e-08f - 0.5f, &sn, &cs); // (-1/2, 1/2)
            const float t = sn / cs;
            d[k] = (srrd == MCIG_SRRD_FISHER) ? signed_by(w[k], 0, t * t) : t;
        }
        return;
    case MCIG_SRRD_EXPONENTIAL:
    case MCIG_SRRD_GAMMA:
    case MCIG_SRRD_WEIBULL:
        for (int k = 0; k < 4; ++k) {
            const float u = ((float)(w[k] >> 8) + 0.5f) * 5.9604644775390625e-08f; // (0, 1)
            d[k] = signed_by(w[k], 0, -logf(u));
        }
        return;
    default: { // LOGNORMAL, CHISQ
        float z[4];
        box_muller_f(q.a, q.b, z[0], z[1]);
        box_muller_f(q.c, q.d, z[2], z[3]);
        for (int k = 0; k < 4; ++k) {
            const float m = (srrd == MCIG_SRRD_LOGNORMAL) ? expf(z[k]) : z[k] * z[k];
            d[k] = signed_by(k < 2 ? q.a : q.c, k & 1, m); // bits 0, 1 of the words whose top 24 bits made u
        }
        return;
    }
    }
}

template <>
__device__ __forceinline__ void move_draws_srrd<double>(P4 q, int srrd, double *d)
{
    switch (srrd) {
    case MCIG_SRRD_UNIFORM: move_draws<double>(q, 0, d); return;
    case MCIG_SRRD_GAUSSIAN: move_draws<double>(q, 1, d); return;
    case MCIG_SRRD_STUDENT:
    case MCIG_SRRD_CAUCHY:
    case MCIG_SRRD_FISHER: {
        const double u[2] = {u01_d(q.a, q.b), u01_d(q.c, q.d)};
        const uint32_t lo[2] = {q.b, q.d};
        for (int k = 0; k < 2; ++k) {
            double sn, cs;
            sincospi((u[k] - 0.5) + 0x1p-54, &sn, &cs); // u in [0, 1): u - 1/2 exact, + 2^-54 in (-1/2, 1/2)
            const double t = sn / cs;
            d[k] = (srrd == MCIG_SRRD_FISHER) ? signed_by(lo[k], 0, t * t) : t;
        }
        return;
    }
    case MCIG_SRRD_EXPONENTIAL:
    case MCIG_SRRD_GAMMA:
    case MCIG_SRRD_WEIBULL:
        d[0] = signed_by(q.b, 0, -log(1.0 - u01_d(q.a, q.b)));
        d[1] = signed_by(q.d, 0, -log(1.0 - u01_d(q.c, q.d)));
        return;
    default: { // LOGNORMAL, CHISQ
        double z0, z1;
        box_muller_d(q, z0, z1);
        d[0] = signed_by(q.b, 0, (srrd == MCIG_SRRD_LOGNORMAL) ? exp(z0) : z0 * z0);
        d[1] = signed_by(q.d, 0, (srrd == MCIG_SRRD_LOGNORMAL) ? exp(z1) : z1 * z1);
        return;
    }
    }
}

template <class R>
__device__ __forceinline__ R accept_draw(P4 q);
// float: on (0, 1], so the log-space test log2(u) <= ... never sees log2(0) = -inf (a
// forced acceptance); double: on [0, 1) with 53 bits, the reference's generate_canonical range
template <>
__device__ __forceinline__ float accept_draw<float>(P4 q) { return u01_open0_f(q.a); }
template <>
__device__ __forceinline__ double accept_draw<double>(P4 q) { return u01_d(q.a, q.b); }

