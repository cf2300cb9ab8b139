// mcig_calib.cuh -- step-size calibration (MCI::findMRT2Step, reference
// src/MCIntegrator.cpp:87-168) of the register-resident float kernel, with the
// calibration's tail split over lanes.
//
// Every chain calibrates on its own (one reference MCI per chain): iterations of
// MIN_STAT steps until the acceptance rate was within 0.05 of the target five times
// in a row, at most |nfind| iterations.  Most chains stop after a few iterations, a
// few run to the limit, so the launch ends with a tail of warps that hold one or two
// running chains each.  A lone warp issues at most one instruction per cycle, so
// that tail lasts as long as the slowest chain's ~40,000 sequential steps at the
// full instruction count of a step.
//
// Phase A runs one chain per lane with the register-resident kernel's step
// (FastSampler::step).  When a warp has at most 32 / LPC running chains left, it
// moves them to phase B: LPC = MAXD / 4 lanes per chain, lane l of a group owning
// coordinates [4l, 4l + 4), i.e. exactly the Philox move block l of the step.  A
// lane draws its block and the step's accept block, moves its four coordinates,
// and the group exchanges the proposal with warp shuffles.  The log density is
// evaluated with the operation order of the one-lane kernel, so phase B gives the
// chain the same numbers bit for bit:
//   exp(-x.x):        every lane sums x_i^2 over the gathered proposal, i ascending;
//   precision matrix: lane l forms the rows {l, 2LPC-1-l, 2LPC+l, 4LPC-1-l} of U x
//                     (upper-triangular U in registers, each row's FMA chain in
//                     ascending column order; the columns left of the diagonal hold
//                     zeros, which leave the chain's +0 start unchanged), then every
//                     lane squares and sums the 4 LPC row values in row order.
// A step of phase B issues about a third of the instructions of a step of phase A,
// so the tail's chains advance about three times faster.
#pragma once

#include "mcig_fast.cuh"

template <int MAXD, int PK>
struct CalibSplit {
    static_assert(MAXD == 16, "the split calibration is instantiated for 16 coordinates");
    static constexpr int LPC = MAXD / 4; // lanes per chain in phase B
    static constexpr int GPW = 32 / LPC; // chains per warp in phase B
    static constexpr int NU = 4 * MAXD - 6 * LPC; // U entries per lane: sum over slots of MAXD - s LPC

    // row of U formed in slot s by lane l: the four slots take rows from the four
    // quarters, alternately ascending and descending, so every lane forms 4 MAXD - 6 LPC
    // products (the rows' lengths MAXD - row balance across the lanes)
    __device__ __forceinline__ static int row(int s, int l) { return (s & 1) ? (s + 1) * LPC - 1 - l : s * LPC + l; }

    // the chain's full coordinate vector from the group's four-coordinate parts
    __device__ __forceinline__ static void gather(const float (&own)[4], float (&full)[MAXD], int base)
    {
#pragma unroll
        for (int i = 0; i < MAXD; ++i) { full[i] = __shfl_sync(0xffffffffu, own[i & 3], base + (i >> 2)); }
    }

    // fast_logp<MAXD, PK> of the full vector xf, with the same operation order
    __device__ __forceinline__ static float logp(const float (&U)[NU], const float (&xf)[MAXD], int base)
    {
        if constexpr (PK == PK_GAUSS) {
            float s = 0.f;
#pragma unroll
            for (int i = 0; i < MAXD; ++i) { s = fmaf(xf[i], xf[i], s); }
            return -s;
        } else {
            float t[4];
            int u = 0;
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                t[s] = 0.f;
#pragma unroll
                for (int j = s * LPC; j < MAXD; ++j) { t[s] = fmaf(U[u++], xf[j], t[s]); }
            }
            float q = 0.f;
#pragma unroll
            for (int i = 0; i < MAXD; ++i) { // row i was formed in slot i / LPC by lane row^-1
                const int s = i / LPC, r = i % LPC;
                const float ti = __shfl_sync(0xffffffffu, t[s], base + ((s & 1) ? LPC - 1 - r : r));
                q = fmaf(ti, ti, q);
            }
            return fast_lp_of_q(q);
        }
    }
};

// MCI::findMRT2Step's step-size update after one iteration (FastSampler::calibrate)
__device__ __forceinline__ void calib_update(const KParams &p, int64_t na, int64_t MIN_STAT, int &cons, float *st)
{
    const double rate = (na > 0) ? (double)na / (double)MIN_STAT : 0.;
    if (fabs(rate - p.target) < 0.05) { ++cons; } else { cons = 0; }
    const double f = fmin(2., fmax(0.5, rate / p.target));
#pragma unroll
    for (int t = 0; t < MCIG_MAXTYPES; ++t) {
        if (t < p.ntypes) {
            double s = (double)st[t] * f;
            double lim = p.step_max;
            for (int i = 0; i < p.ndim; ++i) {
                int tt = 0;
                while (tt + 1 < p.ntypes && i >= p.typeEnds[tt]) { ++tt; }
                if (tt == t && p.step_max_i) { lim = fmin(lim, p.step_max_i[i]); }
            }
            s = fmin(s, lim);
            s = fmax(s, 1.1754943508222875e-38);
            st[t] = (float)s;
        }
    }
}

// the loop condition of findMRT2Step after `counter` iterations with `cons` in a row
__device__ __forceinline__ bool calib_more(const KParams &p, int cons, int counter)
{
    if (p.nfind < 0 && counter >= -p.nfind && counter > 0) { return false; }
    return (p.nfind < 0 && cons < 5) || counter < p.nfind;
}

// Calibration of every chain (KMODE_CALIB): all-coordinate move, one step-size type, no
// periodic domain, a single exp(-x.x) or precision-matrix sampling function.  Results (step
// sizes, walkers, Philox counters, counts of the last iteration) are those of
// FastSampler::calibrate.  Every lane of a warp stays to the end (the warp's shuffles and
// ballots name all 32 lanes); lanes without a chain take no part in the sampling.  LEAN: the
// move's distribution, 1 uniform, 2 Gaussian (FastSampler's LEAN).
template <int MAXD, int PK, int LEAN>
__global__ void __launch_bounds__(MCIG_FAST_BLOCK, 8) mcig_calib_kernel(const KParams p, const FastConst fc)
{
    using CS = CalibSplit<MAXD, PK>;
    constexpr unsigned FULL = 0xffffffffu;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = c < p.nchains && !(p.active && !p.active[c]);
    const int64_t MIN_STAT = p.nsteps;
    FastSampler<MAXD, MCIG_MOVE_ALL, true, PK, false, LEAN> s(p, fc, live ? c : 0, nullptr); // one step type
    int cons = 0, counter = 0;
    int64_t na = 0;
    bool done = !live || !calib_more(p, cons, counter);
    // phase A: one chain per lane while more than GPW chains of the warp run
    for (;;) {
        const unsigned act = __ballot_sync(FULL, !done);
        if (act == 0 || __popc(act) <= CS::GPW) { break; }
        if (!done) {
            s.lp = fast_logp<MAXD, PK>(p, fc, s.x);
            na = 0;
            for (uint32_t r = 0; r < (uint32_t)MIN_STAT; ++r) { na += s.step() ? 1 : 0; }
            calib_update(p, na, MIN_STAT, cons, s.st);
            ++counter;
            done = !calib_more(p, cons, counter);
        }
    }
    if (live && done) {
        s.store_state();
        p.nacc[c] = na;
        p.nrej[c] = (counter > 0) ? MIN_STAT - na : 0;
    }
    const unsigned act = __ballot_sync(FULL, !done);
    if (act == 0) { return; }

    // phase B: group g (lanes [g LPC, g LPC + LPC)) takes the g-th running chain of the warp
    const int lane = threadIdx.x & 31, g = lane / CS::LPC, l = lane % CS::LPC, base = g * CS::LPC;
    unsigned m = act;
    for (int k = 0; k < g && m; ++k) { m &= m - 1; }
    const bool gact = m != 0;
    const int src = gact ? __ffs(m) - 1 : 0; // groups without a chain compute on a copy of lane 0's
    float xo[4];
#pragma unroll
    for (int i = 0; i < MAXD; ++i) {
        const float v = __shfl_sync(FULL, s.x[i], src);
        if ((i >> 2) == l) { xo[i & 3] = v; }
    }
    float st[MCIG_MAXTYPES];
#pragma unroll
    for (int t = 0; t < MCIG_MAXTYPES; ++t) { st[t] = __shfl_sync(FULL, s.st[t], src); }
    uint64_t ctr = ((uint64_t)__shfl_sync(FULL, (uint32_t)(s.ctr >> 32), src) << 32) |
                   (uint64_t)__shfl_sync(FULL, (uint32_t)s.ctr, src);
    const int cc = __shfl_sync(FULL, c, src);
    cons = __shfl_sync(FULL, cons, src);
    counter = __shfl_sync(FULL, counter, src);
    float U[CS::NU];
    if constexpr (PK == PK_PREC) {
        int u = 0;
#pragma unroll
        for (int sl = 0; sl < 4; ++sl) {
            const int r = CS::row(sl, l);
#pragma unroll
            for (int j = sl * CS::LPC; j < MAXD; ++j) { U[u++] = (j >= r) ? fc.fconst[r * MAXD + j] : 0.f; }
        }
    } else {
#pragma unroll
        for (int u = 0; u < CS::NU; ++u) { U[u] = 0.f; }
    }
    float sc[4]; // step sizes of the lane's coordinates (one type: st[0], 0 beyond ndim)
#pragma unroll
    for (int k = 0; k < 4; ++k) { sc[k] = (4 * l + k < p.ndim) ? st[0] : 0.f; }
    constexpr bool gauss = LEAN == 2;
    bool gdone = !gact;
    while (__any_sync(FULL, !gdone)) {
        float xf[MAXD];
        CS::gather(xo, xf, base);
        float lp = CS::logp(U, xf, base);
        na = 0;
        for (uint32_t r = 0; r < (uint32_t)MIN_STAT; ++r) {
            const uint32_t s0 = (uint32_t)ctr, s1 = (uint32_t)(ctr >> 32);
            const P4 qm = philox4x32_10_rk(s0, s1, (uint32_t)cc, (TAG_MOVE << 12) | (uint32_t)l, fc.rk);
            const P4 qa = philox4x32_10_rk(s0, s1, (uint32_t)cc, (TAG_ACCEPT << 12) | 0u, fc.rk);
            float d[4], xn[4];
            move_draws<float>(qm, gauss, d);
#pragma unroll
            for (int k = 0; k < 4; ++k) { xn[k] = fmaf(sc[k], d[k], xo[k]); }
            CS::gather(xn, xf, base);
            const float lpn = CS::logp(U, xf, base);
            if (fast_accept(accept_draw<float>(qa), lpn, lp)) {
#pragma unroll
                for (int k = 0; k < 4; ++k) { xo[k] = xn[k]; }
                lp = lpn;
                ++na;
            }
            ++ctr;
        }
        if (!gdone) {
            calib_update(p, na, MIN_STAT, cons, st);
#pragma unroll
            for (int k = 0; k < 4; ++k) { sc[k] = (4 * l + k < p.ndim) ? st[0] : 0.f; }
            ++counter;
            if (!calib_more(p, cons, counter)) { // the chain's calibration ends: store its state
                gdone = true;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int i = 4 * l + k;
                    if (i < p.ndim) { p.x[(size_t)i * p.nchains + cc] = (double)xo[k]; }
                }
                if (l == 0) {
                    p.step[cc] = (double)st[0];
                    p.ctr[cc] = ctr;
                    p.nacc[cc] = na;
                    p.nrej[cc] = MIN_STAT - na;
                }
            }
        }
    }
}

template <int MAXD, int PK, int LEAN>
void mcig_calib_launch(const KParams &p, const FastConst *fc, int /*movetype*/, int grid, int block, size_t /*smem*/,
                       cudaStream_t st)
{
    mcig_calib_kernel<MAXD, PK, LEAN><<<grid, block, 0, st>>>(p, *fc);
}
