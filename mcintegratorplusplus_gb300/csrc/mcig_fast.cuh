// mcig_fast.cuh -- register-resident float sampling kernel for the common
// configurations: all-coordinate or single-vector moves (uniform / Gaussian),
// any product of sampling functions, observables without exp(), Philox draws.
//
// The walker (x, proposal) lives in registers: MAXD is a compile-time bound on
// ndim and every coordinate loop is unrolled with compile-time indices.  The
// walker is padded to MAXD coordinates whose step size is zero, so no
// coordinate loop carries a predicate.  The sampling-function data (Cholesky
// factor U of a precision matrix with row stride MAXD, mixture parameters) sits
// in the kernel parameter block at fixed offsets, so the unrolled loops take it
// as constant-bank operands without load instructions; the Philox round keys
// are precomputed there too.  Shared memory holds the running sums of
// Simple/Block accumulators, one slot per observable value and thread
// ([slot][thread], conflict-free), float+Kahan or double.
// Full accumulators store every sample straight to HBM, coalesced across the
// warp (layout [nstore][nobs][nchains]).
//
// Semantics are those of the general kernel (mcig_generic.cuh) in float:
// log-space Metropolis test log(u) <= log p(x') - log p(x), one Philox stream
// per chain with the same counter layout, so a chain draws the same uniforms in
// both kernels.
#pragma once

#include "mcig_common.cuh"

#define MCIG_FAST_UNROLLED_OBS 4  // observables handled by the unrolled loop

// log density of the walker (padded to MAXD coordinates with zeros: padded
// coordinates never move, and the parameter data is zero-padded, so no loop
// needs a per-coordinate predicate)
// pdf sets with a kernel of their own: the one-pdf configurations get straight-line
// code for their kind (a runtime switch over every kind would be if-converted and
// issue all of them)
enum { PK_ANY = 0, PK_GAUSS = 1, PK_PREC = 2, PK_MIX = 3 };

// The last operations of the precision-matrix log density and of the Metropolis test,
// shared with the split calibration (mcig_calib.cuh), which evaluates them from the same
// operands in the same expression shape (the compiler's FMA contraction of -q/2 - lp
// is then decided alike; tests/test_fast_accumulators.py checks the bit-identity).
__device__ __forceinline__ float fast_lp_of_q(float q) { return -0.5f * q; }
__device__ __forceinline__ bool fast_accept(float u, float lpn, float lp)
{ // log2(u) <= (log p(x') - log p(x)) log2(e)
    return __log2f(u) <= (lpn - lp) * 1.44269504f;
}

template <int MAXD>
__device__ __forceinline__ float fast_logp_prec(const FastConst &fc, const float *x)
{ // -|U x|^2 / 2, U upper triangular at fconst[0], row stride MAXD
    float q = 0.f;
#pragma unroll
    for (int i = 0; i < MAXD; ++i) {
        float t = 0.f;
#pragma unroll
        for (int j = i; j < MAXD; ++j) { t = fmaf(fc.fconst[i * MAXD + j], x[j], t); }
        q = fmaf(t, t, q);
    }
    return fast_lp_of_q(q);
}

template <int MAXD>
__device__ __forceinline__ float fast_logp_mix(const FastConst &fc, const float *x)
{ // log sum_c exp(lc_c - |(x - m_c) / s_c|^2 / 2) at fconst[MAXD*MAXD], nc <= 8
    constexpr int B = MAXD * MAXD;
    constexpr int S = 1 + 2 * MAXD;
    const int nc = (int)fc.fconst[B];
    float e[8];
    float mx = -INFINITY;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        if (c < nc) {
            float a = 0.f;
#pragma unroll
            for (int i = 0; i < MAXD; ++i) {
                const float z = (x[i] - fc.fconst[B + 1 + c * S + 1 + i]) * fc.fconst[B + 1 + c * S + 1 + MAXD + i];
                a = fmaf(z, z, a);
            }
            a = fmaf(-0.5f, a, fc.fconst[B + 1 + c * S]);
            e[c] = a;
            mx = fmaxf(mx, a);
        }
    }
    float sum = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        if (c < nc) { sum += exp2f((e[c] - mx) * 1.44269504f); }
    }
    return mx + 0.69314718f * __log2f(sum);
}

template <int MAXD, int PK = PK_ANY>
__device__ __forceinline__ float fast_logp(const KParams &p, const FastConst &fc, const float *x)
{
    if constexpr (PK == PK_PREC) { return fast_logp_prec<MAXD>(fc, x); }
    if constexpr (PK == PK_MIX) { return fast_logp_mix<MAXD>(fc, x); }
    if constexpr (PK == PK_GAUSS) { // GAUSS and GAUSS_SUM: -x.x
        float s = 0.f;
#pragma unroll
        for (int i = 0; i < MAXD; ++i) { s = fmaf(x[i], x[i], s); }
        return -s;
    }
    float lp = 0.f;
    for (int k = 0; k < p.npdf; ++k) {
        const PdfDesc &d = p.pdf[k];
        switch (d.kind) {
        case MCIG_PDF_GAUSS_SUM:
        case MCIG_PDF_GAUSS: {
            float s = 0.f;
#pragma unroll
            for (int i = 0; i < MAXD; ++i) { s = fmaf(x[i], x[i], s); }
            lp -= s;
            break;
        }
        case MCIG_PDF_EXP: {
            float s = 0.f;
#pragma unroll
            for (int i = 0; i < MAXD; ++i) { s += fabsf(x[i]); }
            lp -= s;
            break;
        }
        case MCIG_PDF_GAUSS_PREC: lp += fast_logp_prec<MAXD>(fc, x); break;
        case MCIG_PDF_GAUSS_BLOCK: {
            float s = 0.f;
#pragma unroll
            for (int i = 0; i < MAXD; ++i) {
                if (i >= d.b0 && i < d.b1) { s = fmaf(x[i], x[i], s); }
            }
            lp = fmaf(-(float)d.c, s, lp);
            break;
        }
        case MCIG_PDF_GAUSS_MIX: lp += fast_logp_mix<MAXD>(fc, x); break;
        default: break;
        }
    }
    return lp;
}

// n / d for n < 2^31 with the host-computed (magic, shift) of d
__device__ __forceinline__ uint32_t fast_div(uint32_t n, uint32_t magic, uint32_t shift)
{
    return __umulhi(n, magic) >> shift;
}

template <bool KAHAN> struct FastSlot;
template <> struct FastSlot<true> {
    using T = float2;
    __device__ __forceinline__ static void zero(T &v) { v = make_float2(0.f, 0.f); }
    __device__ __forceinline__ static void add(T &v, float a)
    { // Kahan: v.x sum, v.y compensation
        const float y = a - v.y;
        const float t = v.x + y;
        v.y = (t - v.x) - y;
        v.x = t;
    }
    __device__ __forceinline__ static double get(const T &v) { return (double)v.x - (double)v.y; }
};
template <> struct FastSlot<false> {
    using T = double;
    __device__ __forceinline__ static void zero(T &v) { v = 0.; }
    __device__ __forceinline__ static void add(T &v, float a) { v += (double)a; }
    __device__ __forceinline__ static double get(const T &v) { return v; }
};

// MOMENTS: every observable is x (XND) or x.x (X2SUM), Full data in float or a Simple/Block
// accumulator.  The kernel then holds only those paths: the general observable code is a
// runtime choice among every kind and accumulator, which the compiler turns into predicated
// code that issues the arithmetic of all of them on every step; x.x is formed once a step.
// LEAN (1: uniform draws, 2: Gaussian draws): one step-size type and the unbound domain, so
// the step of coordinate i is st[0] (times its 0 / 1 table entry) and the move's distribution
// is known, without the code of the other types, of the other distribution and of the
// periodic wrap: the runtime choices are compiled into predicated code that issues part of
// every alternative on every step (16-D precision-matrix configuration: sampling launch
// 31.3 -> 27.0 ms); 0: general
// FIXED4 (with MOMENTS): exactly one observable in each of the four groups (Full x.x, Full x,
// Simple/Block x.x, Simple/Block x), every nskip 1 and ndim == MAXD: the observable step is one
// straight-line block with no test of its layout
template <int MAXD, int MOVE, bool KAHAN, int PK, bool MOMENTS = false, int LEAN = 0, bool FIXED4 = false>
struct FastSampler {
    using Slot = FastSlot<KAHAN>;
    using ST = typename Slot::T;
    const KParams &p;
    const FastConst &fc;
    const int c;
    ST *slots; // [nobsdim][MCIG_FAST_BLOCK]
    float x[MAXD];
    float st[MCIG_MAXTYPES];
    float lp;
    float xx;   // MOMENTS: x.x of the walker at the current step
    uint32_t s0, s1;
    uint64_t ctr;

    __device__ FastSampler(const KParams &pp, const FastConst &ff, int cc, ST *sl) : p(pp), fc(ff), c(cc), slots(sl)
    {
#pragma unroll
        for (int i = 0; i < MAXD; ++i) { x[i] = (i < p.ndim) ? (float)p.x[(size_t)i * p.nchains + c] : 0.f; }
#pragma unroll
        for (int t = 0; t < MCIG_MAXTYPES; ++t) { st[t] = (t < p.ntypes) ? (float)p.step[(size_t)t * p.nchains + c] : 0.f; }
        ctr = p.ctr[c];
    }

    // step size of coordinate i: st[type(i)], 0 for the padding beyond ndim.  The type
    // table is one-hot in the constant bank, so one step type costs one multiply.
    __device__ __forceinline__ float step_i(int i) const
    {
        float s = st[0] * fc.tw[0][i];
        if constexpr (LEAN != 0) { return s; }
        if (p.ntypes > 1) {
#pragma unroll
            for (int t = 1; t < MCIG_MAXTYPES; ++t) { s = fmaf(st[t], fc.tw[t][i], s); }
        }
        return s;
    }

    __device__ __forceinline__ P4 block(uint32_t tag, uint32_t b) const
    {
        return philox4x32_10_rk(s0, s1, (uint32_t)c, (tag << 12) | b, fc.rk);
    }

    // one Metropolis step (MCI::doStepMRT2, MCIntegrator.cpp:326-360)
    __device__ __forceinline__ bool step()
    {
        s0 = (uint32_t)ctr;
        s1 = (uint32_t)(ctr >> 32);
        const bool gauss = LEAN == 2 ? true : (LEAN == 1 ? false : p.srrd == MCIG_SRRD_GAUSSIAN);
        float xn[MAXD];
        int lo = 0, hi = p.ndim;
        if constexpr (MOVE == MCIG_MOVE_ALL) { // SRRDAllMove::trialMove
#pragma unroll
            for (int b = 0; b < (MAXD + 3) / 4; ++b) {
                float d[4];
                move_draws<float>(block(TAG_MOVE, b), gauss, d);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int i = b * 4 + k;
                    if (i < MAXD) { xn[i] = fmaf(step_i(i), d[k], x[i]); }
                }
            }
        } else { // SRRDVecMove::trialMove
            const int nvecs = p.ndim / p.veclen;
            const int vidx = (int)__umulhi(block(TAG_INDEX, 0).a, (uint32_t)nvecs);
            lo = vidx * p.veclen;
            hi = lo + p.veclen;
#pragma unroll
            for (int b = 0; b < (MAXD + 3) / 4; ++b) {
                float d[4] = {0.f, 0.f, 0.f, 0.f};
                if (b * 4 < hi && b * 4 + 4 > lo) { move_draws<float>(block(TAG_MOVE, b), gauss, d); }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int i = b * 4 + k;
                    if (i < MAXD) { xn[i] = (i >= lo && i < hi) ? fmaf(step_i(i), d[k], x[i]) : x[i]; }
                }
            }
        }
        if (LEAN == 0 && p.periodic) {
#pragma unroll
            for (int i = 0; i < MAXD; ++i) {
                if (i >= lo && i < hi) {
                    const float lb = (float)p.lb[i], ub = (float)p.ub[i], L = ub - lb;
                    int n = 0;
                    while (xn[i] < lb && n < MCIG_PERIODIC_MAXWRAP) { xn[i] += L; ++n; }
                    while (xn[i] > ub && n < MCIG_PERIODIC_MAXWRAP) { xn[i] -= L; ++n; }
                    if (n >= MCIG_PERIODIC_MAXWRAP) { xn[i] = fminf(fmaxf(xn[i], lb), ub); }
                }
            }
        }
        const float lpn = fast_logp<MAXD, PK>(p, fc, xn);
        const float u = accept_draw<float>(block(TAG_ACCEPT, 0));
        const bool acc = fast_accept(u, lpn, lp);
        if (acc) {
#pragma unroll
            for (int i = 0; i < MAXD; ++i) { x[i] = xn[i]; }
            lp = lpn;
        }
        ++ctr;
        return acc;
    }

    __device__ __forceinline__ ST &slot(int j) { return slots[j * MCIG_FAST_BLOCK + threadIdx.x]; }

    // AccumulatorInterface::accumulate of the values v[0..nv) (nv <= NV, compile-time
    // indices) of observable od at accumulation index k.  Full: one coalesced row
    // per value.  Simple/Block: running sums in the shared-memory slots; `flush`
    // marks the last index of block `blk`, whose mean (sum * 1/blocksize) is written
    // and the sums reset (BlockAccumulator.cpp).
    template <int NV>
    __device__ __forceinline__ void put(const ObsDesc &od, uint32_t k, bool flush, uint32_t blk, const float *v, int nv)
    {
        // every value is written (predicate-free) when the observable has NV values,
        // the common case of x and x^2 at ndim == MAXD
        const bool all = (NV == 1) || (nv == NV);
        const uint32_t nc = (uint32_t)p.nchains; // value stride; j * nc < 2^32 for any device array
        if (od.acc == MCIG_ACC_FULL) {
            const size_t row = (size_t)p.acc_offset + k;
            if (od.full32) {
                float *dst = (float *)od.data + row * (size_t)nv * nc + c;
                if (all) {
#pragma unroll
                    for (int j = 0; j < NV; ++j) { dst[j * nc] = v[j]; }
                } else {
#pragma unroll
                    for (int j = 0; j < NV; ++j) {
                        if (j < nv) { dst[j * nc] = v[j]; }
                    }
                }
            } else if constexpr (!MOMENTS) {
                double *dst = (double *)od.data + row * (size_t)nv * nc + c;
#pragma unroll
                for (int j = 0; j < NV; ++j) {
                    if (all || j < nv) { dst[j * nc] = (double)v[j]; }
                }
            }
            return;
        }
        ST *sl = slots + od.voff * MCIG_FAST_BLOCK + threadIdx.x;
        if (all) {
#pragma unroll
            for (int j = 0; j < NV; ++j) { Slot::add(sl[j * MCIG_FAST_BLOCK], v[j]); }
        } else {
#pragma unroll
            for (int j = 0; j < NV; ++j) {
                if (j < nv) { Slot::add(sl[j * MCIG_FAST_BLOCK], v[j]); }
            }
        }
        if (od.acc == MCIG_ACC_BLOCK && flush) {
            double *dst = (double *)od.data + (size_t)blk * nv * nc + c;
#pragma unroll
            for (int j = 0; j < NV; ++j) {
                if (all || j < nv) {
                    dst[j * nc] = Slot::get(sl[j * MCIG_FAST_BLOCK]) * od.inv_bs;
                    Slot::zero(sl[j * MCIG_FAST_BLOCK]);
                }
            }
        }
    }

    // observableFunction of the test classes (oracle obs_eval), in float, then put():
    // the one-value kinds share one put<1>, the vector kinds one put<MAXD>
    __device__ __forceinline__ void observe_put(const ObsDesc &od, uint32_t k, bool flush, uint32_t blk)
    {
        const int kind = od.kind;
        if constexpr (MOMENTS) {
            if (kind == MCIG_OBS_XND) { put<MAXD>(od, k, flush, blk, x, p.ndim); }
            else { put<1>(od, k, flush, blk, &xx, 1); }
            return;
        }
        if (kind == MCIG_OBS_XND || kind == MCIG_OBS_X2 || kind == MCIG_OBS_X2BLOCK) {
            float v[MAXD];
            int nv = p.ndim;
            if (kind == MCIG_OBS_XND) {
#pragma unroll
                for (int i = 0; i < MAXD; ++i) { v[i] = x[i]; }
            } else if (kind == MCIG_OBS_X2) {
#pragma unroll
                for (int i = 0; i < MAXD; ++i) { v[i] = x[i] * x[i]; }
            } else { // X2BLOCK: sum of x_i^2 over each block [b_k, b_k+1)
                const double *pp = p.params + od.poff;
                nv = (int)pp[0];
#pragma unroll
                for (int kb = 0; kb < MAXD; ++kb) {
                    float s = 0.f;
                    if (kb < nv) {
                        const int a = (int)pp[1 + kb], b = (int)pp[2 + kb];
#pragma unroll
                        for (int i = 0; i < MAXD; ++i) {
                            if (i >= a && i < b) { s = fmaf(x[i], x[i], s); }
                        }
                    }
                    v[kb] = s;
                }
            }
            put<MAXD>(od, k, flush, blk, v, nv);
            return;
        }
        float v;
        switch (kind) {
        case MCIG_OBS_X2SUM:
        case MCIG_OBS_X2MEAN: {
            float s = 0.f;
#pragma unroll
            for (int i = 0; i < MAXD; ++i) { s = fmaf(x[i], x[i], s); } // padded coordinates are 0
            v = kind == MCIG_OBS_X2SUM ? s : s / (float)p.ndim;
            break;
        }
        case MCIG_OBS_CONST: v = (float)p.params[od.poff]; break;
        case MCIG_OBS_XI: {
            const int idx = (int)p.params[od.poff];
            v = 0.f;
#pragma unroll
            for (int i = 0; i < MAXD; ++i) { v = (i == idx) ? x[i] : v; }
            break;
        }
        case MCIG_OBS_POLYNOM: {
            v = 0.f;
#pragma unroll
            for (int i = 0; i < MAXD; ++i) { v += x[i]; }
            break;
        }
        case MCIG_OBS_LOGPDF: v = lp; break; // the log density the Metropolis test keeps for the walker
        default: return;
        }
        put<1>(od, k, flush, blk, &v, 1);
    }

    // observable od after step r: accumulation index k = r / nskip when nskip
    // divides r (AccumulatorInterface.cpp:31-60), block end when blocksize divides k + 1
    __device__ __forceinline__ void obs_step(const ObsDesc &od, uint32_t r)
    {
        uint32_t k = r;
        if (od.nskip != 1) {
            k = fast_div(r, od.sk_magic, od.sk_shift);
            if (k * (uint32_t)od.nskip != r) { return; }
        }
        uint32_t blk = 0;
        bool flush = false;
        if (od.acc == MCIG_ACC_BLOCK) {
            const uint32_t q = fast_div(k + 1, od.bs_magic, od.bs_shift);
            flush = q * (uint32_t)od.bs == k + 1;
            blk = q - 1;
        }
        observe_put(od, k, flush, blk);
    }

    // MOMENTS: observable od of a group whose accumulator (Full or Simple/Block) and kind (x or
    // x.x) are known at compile time, after step r (the accumulation index and block end of
    // obs_step; Full data in float).  Without the general code's runtime choice of kind and
    // accumulator per observable, the step issues only the chosen path.
    template <bool FULL, bool VEC>
    __device__ __forceinline__ void obs_group_one(const ObsDesc &od, uint32_t r)
    {
        constexpr int NV = VEC ? MAXD : 1;
        uint32_t k = r;
        if (!FIXED4 && od.nskip != 1) {
            k = fast_div(r, od.sk_magic, od.sk_shift);
            if (k * (uint32_t)od.nskip != r) { return; }
        }
        const uint32_t nc = (uint32_t)p.nchains; // value stride; j * nc < 2^32 for any device array
        const float *v = VEC ? x : &xx;
        const bool all = FIXED4 || !VEC || p.ndim == MAXD; // every value exists: no predicate per value
        if constexpr (FULL) {
            float *dst = (float *)od.data + ((size_t)p.acc_offset + k) * (size_t)od.nv * nc + c;
            if (all) {
#pragma unroll
                for (int j = 0; j < NV; ++j) { dst[j * nc] = v[j]; }
            } else {
#pragma unroll
                for (int j = 0; j < NV; ++j) {
                    if (j < od.nv) { dst[j * nc] = v[j]; }
                }
            }
        } else {
            ST *sl = slots + od.voff * MCIG_FAST_BLOCK + threadIdx.x;
            if (all) {
#pragma unroll
                for (int j = 0; j < NV; ++j) { Slot::add(sl[j * MCIG_FAST_BLOCK], v[j]); }
            } else {
#pragma unroll
                for (int j = 0; j < NV; ++j) {
                    if (j < od.nv) { Slot::add(sl[j * MCIG_FAST_BLOCK], v[j]); }
                }
            }
            if (od.acc == MCIG_ACC_BLOCK) {
                const uint32_t q = fast_div(k + 1, od.bs_magic, od.bs_shift);
                if (q * (uint32_t)od.bs == k + 1) { // block end: mean of the block, sums reset
                    double *dst = (double *)od.data + (size_t)(q - 1) * od.nv * nc + c;
#pragma unroll
                    for (int j = 0; j < NV; ++j) {
                        if (all || j < od.nv) {
                            dst[j * nc] = Slot::get(sl[j * MCIG_FAST_BLOCK]) * od.inv_bs;
                            Slot::zero(sl[j * MCIG_FAST_BLOCK]);
                        }
                    }
                }
            }
        }
    }

    // MOMENTS: every observable after step r, group by group (FastSampler's launcher orders
    // them).  With at most one observable per group (mgroup[4] == 1 marks that layout; the
    // launcher then puts group g's observable, if any, at obs[g]) the groups are straight-line
    // code over descriptors at fixed parameter offsets (constant-bank operands); otherwise
    // loops over each group.
    __device__ __forceinline__ void obs_groups(uint32_t r)
    {
        if (p.mgroup_slots) {
            if (p.mgroup[0]) { obs_group_one<true, false>(p.obs[0], r); }
            if (p.mgroup[1]) { obs_group_one<true, true>(p.obs[1], r); }
            if (p.mgroup[2]) { obs_group_one<false, false>(p.obs[2], r); }
            if (p.mgroup[3]) { obs_group_one<false, true>(p.obs[3], r); }
            return;
        }
        int o = 0;
        for (int i = 0; i < p.mgroup[0]; ++i, ++o) { obs_group_one<true, false>(p.obs[o], r); }
        for (int i = 0; i < p.mgroup[1]; ++i, ++o) { obs_group_one<true, true>(p.obs[o], r); }
        for (int i = 0; i < p.mgroup[2]; ++i, ++o) { obs_group_one<false, false>(p.obs[o], r); }
        for (int i = 0; i < p.mgroup[3]; ++i, ++o) { obs_group_one<false, true>(p.obs[o], r); }
    }

    // n < 2^32 (checked on the host); accumulation indices in 32-bit arithmetic.
    // The first MCIG_FAST_UNROLLED_OBS observables are unrolled, so their
    // descriptors are constant-bank operands; any further ones loop.
    __device__ void run(int64_t n, bool sample)
    {
        lp = fast_logp<MAXD, PK>(p, fc, x);
        for (int j = 0; j < p.nobsdim && sample; ++j) { Slot::zero(slot(j)); }
        const uint32_t n32 = (uint32_t)n;
        const uint32_t r0 = (uint32_t)p.r0; // chunked sampling: global index of the first step
        uint32_t na = 0;
        for (uint32_t r = 0; r < n32; ++r) {
            na += step() ? 1u : 0u;
            if (!sample) { continue; }
            if constexpr (MOMENTS) { // the X2SUM value of the general path, formed once
                float s = 0.f;
#pragma unroll
                for (int i = 0; i < MAXD; ++i) { s = fmaf(x[i], x[i], s); }
                xx = s;
                if constexpr (FIXED4) {
                    obs_group_one<true, false>(p.obs[0], r0 + r);
                    obs_group_one<true, true>(p.obs[1], r0 + r);
                    obs_group_one<false, false>(p.obs[2], r0 + r);
                    obs_group_one<false, true>(p.obs[3], r0 + r);
                } else {
                    obs_groups(r0 + r);
                }
                continue;
            }
#pragma unroll
            for (int o = 0; o < MCIG_FAST_UNROLLED_OBS; ++o) {
                if (o < p.nobs) { obs_step(p.obs[o], r0 + r); }
            }
            for (int o = MCIG_FAST_UNROLLED_OBS; o < p.nobs; ++o) { obs_step(p.obs[o], r0 + r); }
        }
        if (sample) {
            for (int o = 0; o < p.nobs; ++o) { // SimpleAccumulator::_finalize
                const ObsDesc &od = p.obs[o];
                if (od.acc != MCIG_ACC_SIMPLE) { continue; }
                const double normf = 1. / (double)(1 + (n - 1) / od.nskip);
                double *dst = (double *)od.data + c;
                for (int j = 0; j < od.nv; ++j) { dst[(size_t)j * p.nchains] = Slot::get(slot(od.voff + j)) * normf; }
            }
        }
        if (p.acc_counts) {
            p.nacc[c] += na;
            p.nrej[c] += n - na;
        } else {
            p.nacc[c] = na;
            p.nrej[c] = n - na;
        }
    }

    // MCI::findMRT2Step (MCIntegrator.cpp:87-168) for this chain alone
    __device__ void calibrate(int64_t MIN_STAT)
    {
        int cons = 0, counter = 0;
        int64_t na = 0;
        while ((p.nfind < 0 && cons < 5) || counter < p.nfind) {
            lp = fast_logp<MAXD, PK>(p, fc, x);
            na = 0;
            for (uint32_t r = 0; r < (uint32_t)MIN_STAT; ++r) { na += step() ? 1 : 0; }
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
            ++counter;
            if (p.nfind < 0 && counter >= abs(p.nfind)) { break; }
        }
        p.nacc[c] = na;
        p.nrej[c] = (counter > 0) ? MIN_STAT - na : 0;
    }

    __device__ void store_state()
    {
#pragma unroll
        for (int i = 0; i < MAXD; ++i) {
            if (i < p.ndim) { p.x[(size_t)i * p.nchains + c] = (double)x[i]; }
        }
#pragma unroll
        for (int t = 0; t < MCIG_MAXTYPES; ++t) {
            if (t < p.ntypes) { p.step[(size_t)t * p.nchains + c] = (double)st[t]; }
        }
        p.ctr[c] = ctr;
    }
};

// Up to 16 dimensions the kernel is held to 128 registers per thread: registers are
// allocated in steps that make 136 or 144 per thread fit only six 64-thread blocks
// per SM (912 of the 1,024 blocks of 65,536 chains, so a second wave), 128 fits eight.
template <int MAXD, int MOVE, bool KAHAN, int PK, bool MOMENTS = false, int LEAN = 0, bool FIXED4 = false>
__global__ void __launch_bounds__(MCIG_FAST_BLOCK, MAXD <= 16 ? 8 : 2) mcig_fast_kernel(const KParams p, const FastConst fc)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using ST = typename FastSlot<KAHAN>::T;
    ST *slots = (ST *)smem_raw;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= p.nchains) { return; }
    if (p.active && !p.active[c]) { return; }
    FastSampler<MAXD, MOVE, KAHAN, PK, MOMENTS, LEAN, FIXED4> s(p, fc, c, slots);
    if (p.mode == KMODE_CALIB) { s.calibrate(p.nsteps); }
    else if (p.mode == KMODE_FUSED) {
        // MCI::integrate's phases for this chain alone: a chain whose calibration converges
        // early goes on sampling while the others still calibrate
        if (p.fuse_calib > 0) { s.calibrate(p.fuse_calib); }
        if (p.fuse_burnin > 0) { s.run(p.fuse_burnin, false); }
        s.run(p.nsteps, true);
    } else {
        s.run(p.nsteps, p.mode == KMODE_SAMPLE);
    }
    s.store_state();
}

template <int MAXD, int MOVE, bool KAHAN, int PK = PK_ANY, bool MOMENTS = false, int LEAN = 0, bool FIXED4 = false>
void mcig_fast_launch(const KParams &p, const FastConst *fc, int /*movetype*/, int grid, int block, size_t smem,
                      cudaStream_t st)
{
    auto k = mcig_fast_kernel<MAXD, MOVE, KAHAN, PK, MOMENTS, LEAN, FIXED4>;
    // shared memory as large as possible, so the accumulator slots never limit residency
    mcig_smem_attrs((const void *)k, smem);
    if constexpr (MOMENTS) { // the observables in four groups (KParams::mgroup), order kept within each
        KParams q = p;
        int n = 0, most = 0;
        for (int g = 0; g < 4; ++g) {
            q.mgroup[g] = 0;
            for (int o = 0; o < p.nobs; ++o) {
                const ObsDesc &od = p.obs[o];
                const int og = (od.acc == MCIG_ACC_FULL ? 0 : 2) + (od.kind == MCIG_OBS_XND ? 1 : 0);
                if (og == g) {
                    q.obs[n++] = od;
                    ++q.mgroup[g];
                }
            }
            most = q.mgroup[g] > most ? q.mgroup[g] : most;
        }
        q.mgroup_slots = most <= 1;
        if (q.mgroup_slots) { // group g's observable at obs[g] (the Simple finalize reads every slot < nobs)
            KParams r = q;
            int o = 0;
            for (int g = 0; g < 4; ++g) {
                if (q.mgroup[g]) { r.obs[g] = q.obs[o++]; }
                else { r.obs[g] = ObsDesc{}; r.obs[g].acc = -1; }
            }
            r.nobs = 4;
            q = r;
        }
        k<<<grid, block, smem, st>>>(q, *fc);
        return;
    }
    k<<<grid, block, smem, st>>>(p, *fc);
}
