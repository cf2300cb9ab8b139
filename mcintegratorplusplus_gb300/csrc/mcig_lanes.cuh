// mcig_lanes.cuh -- float sampling kernel with LPC lanes per chain for a mixture of
// Gaussians (one GAUSS_MIX sampling function, all-coordinate move, one step type,
// unbound domain): the precision form's workload, 16,384 chains of a 32-D mixture of 8.
//
// One lane per chain (mcig_fast.cuh) leaves a GPU of 152 SMs with 3.4 warps per SM at
// 16,384 chains, too few to hide the latency of the mixture's dependent arithmetic.  Here
// the LPC lanes of a chain share its work:
//   * lane group l owns coordinates [l CPL, (l+1) CPL), CPL = MAXD / LPC, i.e. the Philox
//     move blocks l CPL / 4 ... of the step: it draws and moves only its coordinates;
//   * the proposal's coordinates reach every lane by warp shuffles, a pair at a time, and
//     lane group l adds them into mixture components l, l + LPC, ..., each component's sum
//     in ascending coordinate order (the one-lane kernel's order);
//   * the maximum over components is a butterfly over the chain's lanes (exact), each lane
//     exponentiates its own components, and every lane sums the gathered terms in
//     component order.
// The log density, the Metropolis decision, the walker and the accumulators are therefore
// those of the one-lane kernel bit for bit (tests/test_lanes.py); only the time changes.
// Lane layout in a warp: lane = l * G + k, G = 32 / LPC chains per warp, so the lanes of
// one group hold G consecutive chains and their Full stores are contiguous.
//
// Certified FP64 decision (the precision form's "FP64 for the log-acceptance ratio"):
// with KParams::f64_decide == 1 the float test log2(u) <= (lp' - lp) log2(e) decides unless
// |log2(u) - (lp' - lp) log2(e)| is below the float evaluation's error margin
//   tol = (2^-12 + 2^-18 (|lp| + |lp'|)) log2(e),
// about seven times the bound of the float mixture's rounding (32 squared terms with
// relative rounding 2^-24 each, exp2/log2 of terms <= 1); inside it, the log densities of
// the walker and the proposal (both exactly representable float positions) are evaluated
// in double with the reference's formula and log(u) <= log p(x') - log p(x) decides in
// double.  The decision is then the one an FP64 evaluation of the same positions takes.
// f64_decide == 2 evaluates the double test on every step (a diagnostic: the counters
// KParams::dstats record how many float decisions the double test reversed and the largest
// float margin among them, which must stay below tol).  The walk is in log space, so no
// acceptance underflows; a proposal with log p(x') - log p(x) < -17 is never accepted by a
// 24-bit uniform (u >= 2^-24), the double test keeps that.
#pragma once

#include "mcig_calib.cuh"

// own coordinates of a lane, passed by value to the out-of-line double decision
template <int CPL> struct LaneVec { float v[CPL]; };

// The Metropolis decision in double for the chain of this lane (every lane of the warp
// calls it: the walker and the proposal are gathered with shuffles): log(u) <= log p(x') -
// log p(x) at the float positions x (own part xo) and x' (own part xno), log p in double by
// the reference formula of the double kernels' pdf_proto_scalar_d and of the oracle, with
// pp = [nc, w[nc], m[nc][nd], s[nc][nd], lc[nc]]:
//   e_q = lc_q + sum_i -0.5 ((x_i - m_qi) / s_qi)^2 (ascending i), M = max_q e_q,
//   log p = M + log(sum_q exp(e_q - M)) (ascending q).
// The chain's LPC lanes share it as the float path shares the float mixture: lane group l
// evaluates components l, l + LPC, ..., the maximum is a butterfly over the chain's lanes
// (exact), and every lane sums the gathered terms in component order, so each lane computes
// nc / LPC components instead of all of them, with the same result bit for bit.  Out of
// line, so that the rare double path takes no registers from the sampling loop.
template <int MAXD, int LPC>
__device__ __noinline__ bool lanes_decide_d(const double *pp, int nd, int nc, int l, int k, float u,
                                            LaneVec<MAXD / LPC> xo, LaneVec<MAXD / LPC> xno)
{
    constexpr int CPL = MAXD / LPC, G = 32 / LPC, CPP = 8 / LPC;
    constexpr unsigned FULL = 0xffffffffu;
    double xd[MAXD], xnd[MAXD];
#pragma unroll
    for (int i = 0; i < MAXD; ++i) {
        xd[i] = (double)__shfl_sync(FULL, xo.v[i % CPL], (i / CPL) * G + k);
        xnd[i] = (double)__shfl_sync(FULL, xno.v[i % CPL], (i / CPL) * G + k);
    }
    const double *m = pp + 1 + nc, *sg = pp + 1 + nc + nc * nd, *lc = pp + 1 + nc + 2 * nc * nd;
    double eo[CPP], en[CPP];
    double mo = -INFINITY, mn = -INFINITY;
#pragma unroll
    for (int r = 0; r < CPP; ++r) {
        const int q = l + LPC * r;
        double a = -INFINITY, b = -INFINITY;
        if (q < nc) {
            a = lc[q];
            b = lc[q];
            for (int i = 0; i < nd; ++i) {
                const double zo = (xd[i] - m[q * nd + i]) / sg[q * nd + i];
                a += -0.5 * (zo * zo);
                const double zn = (xnd[i] - m[q * nd + i]) / sg[q * nd + i];
                b += -0.5 * (zn * zn);
            }
        }
        eo[r] = a;
        en[r] = b;
        mo = a > mo ? a : mo;
        mn = b > mn ? b : mn;
    }
#pragma unroll
    for (int s = G; s < 32; s <<= 1) {
        const double oo = __shfl_xor_sync(FULL, mo, s), on = __shfl_xor_sync(FULL, mn, s);
        mo = oo > mo ? oo : mo;
        mn = on > mn ? on : mn;
    }
    double to[CPP], tn[CPP];
#pragma unroll
    for (int r = 0; r < CPP; ++r) {
        to[r] = (l + LPC * r < nc) ? exp(eo[r] - mo) : 0.;
        tn[r] = (l + LPC * r < nc) ? exp(en[r] - mn) : 0.;
    }
    double so = 0., sn = 0.;
#pragma unroll
    for (int q = 0; q < 8; ++q) { // component q sits in lane group q % LPC, slot q / LPC
        const double a = __shfl_sync(FULL, to[q / LPC], (q % LPC) * G + k);
        const double b = __shfl_sync(FULL, tn[q / LPC], (q % LPC) * G + k);
        if (q < nc) {
            so += a;
            sn += b;
        }
    }
    return log((double)u) <= (mn + log(sn)) - (mo + log(so));
}

template <int MAXD, int LPC, bool KAHAN, bool GAUSS = true> // GAUSS: Gaussian (else uniform) move draws
struct LaneMixSampler {
    static_assert(MAXD % (4 * LPC) == 0 && 32 % LPC == 0 && LPC >= 2 && LPC <= 8, "lanes own whole Philox blocks");
    static constexpr int CPL = MAXD / LPC;         // coordinates per lane
    static constexpr int BPL = CPL / 4;            // Philox move blocks per lane
    static constexpr int G = 32 / LPC;             // chains per warp
    static constexpr int CPP = 8 / LPC;            // mixture components per lane (<= 8 components)
    static constexpr int TS = MAXD / 2 + 1;        // float4 per component row of the table (+1: banks)
    static constexpr unsigned FULL = 0xffffffffu;
    using Slot = FastSlot<KAHAN>;
    using ST = typename Slot::T;

    const KParams &p;
    const FastConst &fc;
    const float4 *tab;   // [8][TS]: (m_i, 1/s_i, m_i+1, 1/s_i+1)
    const float *lcn;    // [8] log normalisation of each component
    ST *slots;           // [nslot][blockDim.x]
    int nc;              // components
    int l, k, c;         // coordinate group, chain in warp, chain
    bool valid;          // a chain of this launch
    float x[CPL], sto[CPL];
    float st[MCIG_MAXTYPES];
    float lp, xx, sx;    // log density, x.x and sum x_i of the walker
    uint64_t ctr;
    bool need_xx, need_sx;

    __device__ static bool vec_kind(int kind) { return kind == MCIG_OBS_XND || kind == MCIG_OBS_X2; }

    __device__ LaneMixSampler(const KParams &pp, const FastConst &ff, const float4 *tb, const float *lc, ST *sl,
                              int lane_group, int chain_in_warp, int chain)
        : p(pp), fc(ff), tab(tb), lcn(lc), slots(sl), l(lane_group), k(chain_in_warp), c(chain)
    {
        nc = (int)fc.fconst[MAXD * MAXD];
        valid = c < p.nchains && (!p.active || p.active[c]);
        const int cc = c < p.nchains ? c : 0;
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            const int i = l * CPL + m;
            x[m] = (valid && i < p.ndim) ? (float)p.x[(size_t)i * p.nchains + cc] : 0.f;
        }
#pragma unroll
        for (int t = 0; t < MCIG_MAXTYPES; ++t) { st[t] = (valid && t < p.ntypes) ? (float)p.step[(size_t)t * p.nchains + cc] : 0.f; }
        set_steps();
        ctr = valid ? p.ctr[cc] : 0;
        need_xx = need_sx = false;
        for (int o = 0; o < p.nobs; ++o) {
            const int kind = p.obs[o].kind;
            need_xx |= kind == MCIG_OBS_X2SUM || kind == MCIG_OBS_X2MEAN;
            need_sx |= kind == MCIG_OBS_POLYNOM;
        }
    }

    // step of the own coordinates: st[0] (one step type), 0 for the padding beyond ndim
    // (the one-lane kernel's step_i with a one-hot type table: st[0] * 1 or * 0)
    __device__ __forceinline__ void set_steps()
    {
#pragma unroll
        for (int m = 0; m < CPL; ++m) { sto[m] = (l * CPL + m < p.ndim) ? st[0] : 0.f; }
    }

    // fast_logp_mix<MAXD> of the chain's vector whose own coordinates this lane holds in
    // `own`, same operation order; the coordinates are gathered one pair at a time as the
    // component sums consume them (no MAXD-register copy of the vector), and x.x and the sum
    // of the coordinates (one-lane order: i ascending) are formed in the same pass
    __device__ __forceinline__ float logp(const float (&own)[CPL], float &xxo, float &sxo) const
    {
        float a[CPP];
#pragma unroll
        for (int r = 0; r < CPP; ++r) { a[r] = 0.f; }
        float xx2 = 0.f, sx2 = 0.f;
#pragma unroll
        for (int i = 0; i < MAXD; i += 2) {
            // at most 8 table loads in flight: the compiler would otherwise hoist all of
            // them (4 registers each) and spill
            if (i % 16 == 0) { asm volatile("" ::: "memory"); }
            const float x0 = __shfl_sync(FULL, own[i % CPL], (i / CPL) * G + k);
            const float x1 = __shfl_sync(FULL, own[(i + 1) % CPL], ((i + 1) / CPL) * G + k);
#pragma unroll
            for (int r = 0; r < CPP; ++r) {
                const float4 t = tab[(l + LPC * r) * TS + i / 2];
                float z = (x0 - t.x) * t.y;
                a[r] = fmaf(z, z, a[r]);
                z = (x1 - t.z) * t.w;
                a[r] = fmaf(z, z, a[r]);
            }
            if (need_xx) {
                xx2 = fmaf(x0, x0, xx2);
                xx2 = fmaf(x1, x1, xx2);
            }
            if (need_sx) {
                sx2 += x0;
                sx2 += x1;
            }
        }
        xxo = xx2;
        sxo = sx2;
        float e[CPP];
        float mx = -INFINITY;
#pragma unroll
        for (int r = 0; r < CPP; ++r) {
            const int cc = l + LPC * r;
            e[r] = (cc < nc) ? fmaf(-0.5f, a[r], lcn[cc]) : -INFINITY;
            mx = fmaxf(mx, e[r]);
        }
#pragma unroll
        for (int s = G; s < 32; s <<= 1) { mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, s)); }
        float term[CPP];
#pragma unroll
        for (int r = 0; r < CPP; ++r) { term[r] = exp2f((e[r] - mx) * 1.44269504f); }
        float sum = 0.f;
#pragma unroll
        for (int cc = 0; cc < 8; ++cc) { // component cc sits in lane group cc % LPC, slot cc / LPC
            const float t = __shfl_sync(FULL, term[cc / LPC], (cc % LPC) * G + k);
            if (cc < nc) { sum += t; }
        }
        return mx + 0.69314718f * __log2f(sum);
    }

    // the Metropolis decision, certified against double near the threshold (see the header)
    __device__ __forceinline__ bool decide(float u, float lpn, const float (&xn)[CPL], bool upd)
    {
        const float l2u = __log2f(u), dl2 = (lpn - lp) * 1.44269504f;
        bool acc = l2u <= dl2; // fast_accept(u, lpn, lp)
        if (p.f64_decide) {
            const float tol2 = (0x1p-12f + 0x1p-18f * (fabsf(lp) + fabsf(lpn))) * 1.44269504f;
            const bool near = valid && upd && (p.f64_decide == 2 || fabsf(l2u - dl2) < tol2);
            if (__any_sync(FULL, near)) {
                LaneVec<CPL> xo, xno;
#pragma unroll
                for (int m = 0; m < CPL; ++m) {
                    xo.v[m] = x[m];
                    xno.v[m] = xn[m];
                }
                const bool a64 = lanes_decide_d<MAXD, LPC>(p.params + p.pdf[0].poff, p.ndim, nc, l, k, u, xo, xno);
                if (near) {
                    if (p.dstats && l == 0) {
                        atomicAdd(p.dstats, 1ull);
                        if (a64 != acc) {
                            atomicAdd(p.dstats + 1, 1ull);
                            atomicMax(p.dstats + 2, (unsigned long long)__float_as_uint(fabsf(l2u - dl2) * 0.69314718f));
                        }
                    }
                    acc = a64;
                }
            }
        }
        return acc;
    }

    // one Metropolis step (MCI::doStepMRT2); upd false: the chain takes no part (the lanes
    // still join the shuffles)
    __device__ __forceinline__ bool step(bool upd)
    {
        const uint32_t s0 = (uint32_t)ctr, s1 = (uint32_t)(ctr >> 32);
        constexpr bool gauss = GAUSS;
        float xn[CPL];
#pragma unroll
        for (int j = 0; j < BPL; ++j) {
            float d[4];
            move_draws<float>(philox4x32_10_rk(s0, s1, (uint32_t)c, (TAG_MOVE << 12) | (uint32_t)(l * BPL + j), fc.rk), gauss, d);
#pragma unroll
            for (int i = 0; i < 4; ++i) { xn[4 * j + i] = fmaf(sto[4 * j + i], d[i], x[4 * j + i]); }
        }
        float xxn, sxn;
        const float lpn = logp(xn, xxn, sxn);
        const float u = accept_draw<float>(philox4x32_10_rk(s0, s1, (uint32_t)c, TAG_ACCEPT << 12, fc.rk));
        const bool acc = decide(u, lpn, xn, upd);
        if (upd) {
            if (acc) {
#pragma unroll
                for (int m = 0; m < CPL; ++m) { x[m] = xn[m]; }
                lp = lpn;
                xx = xxn;
                sx = sxn;
            }
            ++ctr;
        }
        return upd && acc;
    }

    // the walker's log density and sums, evaluated as the one-lane kernel does at a start
    __device__ __forceinline__ void refresh() { lp = logp(x, xx, sx); }

    __device__ __forceinline__ ST &slot(int j) { return slots[j * blockDim.x + threadIdx.x]; }

    // AccumulatorInterface::accumulate of value j (index in the observable) at accumulation k
    __device__ __forceinline__ void put1(const ObsDesc &od, int s, int j, uint32_t kk, bool flush, uint32_t blk, float v)
    {
        const uint32_t ncs = (uint32_t)p.nchains;
        if (od.acc == MCIG_ACC_FULL) {
            const size_t row = (size_t)p.acc_offset + kk;
            if (od.full32) { ((float *)od.data)[(row * (size_t)od.nv + j) * ncs + c] = v; }
            else { ((double *)od.data)[(row * (size_t)od.nv + j) * ncs + c] = (double)v; }
            return;
        }
        ST &sl = slot(s);
        Slot::add(sl, v);
        if (od.acc == MCIG_ACC_BLOCK && flush) {
            ((double *)od.data)[((size_t)blk * od.nv + j) * ncs + c] = Slot::get(sl) * od.inv_bs;
            Slot::zero(sl);
        }
    }

    __device__ __forceinline__ void observe(const ObsDesc &od, uint32_t kk, bool flush, uint32_t blk)
    {
        const int kind = od.kind;
        if (vec_kind(kind)) {
#pragma unroll
            for (int m = 0; m < CPL; ++m) {
                const int j = l * CPL + m;
                const float v = kind == MCIG_OBS_XND ? x[m] : x[m] * x[m];
                if (valid && j < od.nv) { put1(od, od.lslot + m, j, kk, flush, blk, v); }
            }
            return;
        }
        float v = 0.f;
        if (kind == MCIG_OBS_XI) { // the lane group holding coordinate idx hands it to group 0
            const int idx = (int)p.params[od.poff];
            const int mi = idx % CPL;
            float mine = 0.f;
#pragma unroll
            for (int m = 0; m < CPL; ++m) { mine = (m == mi) ? x[m] : mine; }
            v = __shfl_sync(FULL, mine, (idx / CPL) * G + k);
        } else if (kind == MCIG_OBS_X2SUM) {
            v = xx;
        } else if (kind == MCIG_OBS_X2MEAN) {
            v = xx / (float)p.ndim;
        } else if (kind == MCIG_OBS_CONST) {
            v = (float)p.params[od.poff];
        } else if (kind == MCIG_OBS_POLYNOM) {
            v = sx;
        } else if (kind == MCIG_OBS_LOGPDF) {
            v = lp;
        }
        if (valid && l == 0) { put1(od, od.lslot, 0, kk, flush, blk, v); }
    }

    __device__ __forceinline__ void obs_step(const ObsDesc &od, uint32_t r)
    {
        uint32_t kk = r;
        if (od.nskip != 1) {
            kk = fast_div(r, od.sk_magic, od.sk_shift);
            if (kk * (uint32_t)od.nskip != r) { return; }
        }
        uint32_t blk = 0;
        bool flush = false;
        if (od.acc == MCIG_ACC_BLOCK) {
            const uint32_t q = fast_div(kk + 1, od.bs_magic, od.bs_shift);
            flush = q * (uint32_t)od.bs == kk + 1;
            blk = q - 1;
        }
        observe(od, kk, flush, blk);
    }

    __device__ __forceinline__ void run(int64_t n, bool sample)
    {
        refresh();
        int nslot = 0;
        for (int o = 0; o < p.nobs; ++o) { nslot += vec_kind(p.obs[o].kind) ? CPL : 1; }
        for (int j = 0; j < nslot && sample; ++j) { Slot::zero(slot(j)); }
        const uint32_t n32 = (uint32_t)n;
        uint32_t na = 0;
        for (uint32_t r = 0; r < n32; ++r) {
            na += step(valid) ? 1u : 0u;
            if (!sample) { continue; }
#pragma unroll
            for (int o = 0; o < MCIG_FAST_UNROLLED_OBS; ++o) {
                if (o < p.nobs) { obs_step(p.obs[o], r); }
            }
            for (int o = MCIG_FAST_UNROLLED_OBS; o < p.nobs; ++o) { obs_step(p.obs[o], r); }
        }
        if (sample && valid) {
            for (int o = 0; o < p.nobs; ++o) { // SimpleAccumulator::_finalize
                const ObsDesc &od = p.obs[o];
                if (od.acc != MCIG_ACC_SIMPLE) { continue; }
                const double normf = 1. / (double)(1 + (n - 1) / od.nskip);
                double *dst = (double *)od.data + c;
                if (vec_kind(od.kind)) {
                    for (int m = 0; m < CPL; ++m) {
                        const int j = l * CPL + m;
                        if (j < od.nv) { dst[(size_t)j * p.nchains] = Slot::get(slot(od.lslot + m)) * normf; }
                    }
                } else if (l == 0) {
                    dst[0] = Slot::get(slot(od.lslot)) * normf;
                }
            }
        }
        if (valid && l == 0) {
            p.nacc[c] = na;
            p.nrej[c] = n - na;
        }
    }

    // MCI::findMRT2Step (MCIntegrator.cpp:87-168) for every chain of the warp, each on its
    // own (FastSampler::calibrate's loop); the warp runs until its last chain has finished
    __device__ __forceinline__ void calibrate(int64_t MIN_STAT)
    {
        int cons = 0, counter = 0;
        int64_t na = 0;
        bool runc = valid && calib_more(p, cons, counter);
        while (__any_sync(FULL, runc)) {
            {
                float xx0, sx0;
                const float l0 = logp(x, xx0, sx0);
                if (runc) { lp = l0; }
            }
            int64_t nacc = 0;
            for (uint32_t r = 0; r < (uint32_t)MIN_STAT; ++r) { nacc += step(runc) ? 1 : 0; }
            if (runc) {
                na = nacc;
                calib_update(p, na, MIN_STAT, cons, st);
                set_steps();
                ++counter;
                runc = calib_more(p, cons, counter);
            }
        }
        if (valid && l == 0) {
            p.nacc[c] = na;
            p.nrej[c] = (counter > 0) ? MIN_STAT - na : 0;
        }
    }

    __device__ __forceinline__ void store_state()
    {
        if (!valid) { return; }
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            const int i = l * CPL + m;
            if (i < p.ndim) { p.x[(size_t)i * p.nchains + c] = (double)x[m]; }
        }
        if (l == 0) {
#pragma unroll
            for (int t = 0; t < MCIG_MAXTYPES; ++t) {
                if (t < p.ntypes) { p.step[(size_t)t * p.nchains + c] = (double)st[t]; }
            }
            p.ctr[c] = ctr;
        }
    }
};

// shared memory of a launch: the component table and the lanes' accumulator slots
template <int MAXD>
struct LanesTable { static constexpr size_t bytes = (size_t)8 * (MAXD / 2 + 1) * sizeof(float4) + 8 * sizeof(float); };

template <int MAXD, int LPC, bool KAHAN, bool GAUSS>
__global__ void __launch_bounds__(MCIG_FAST_BLOCK, LPC >= 8 ? 14 : 8) mcig_lanes_kernel(const KParams p, const FastConst fc)
{
    using LS = LaneMixSampler<MAXD, LPC, KAHAN, GAUSS>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4 *tab = (float4 *)smem_raw;
    float *lcn = (float *)(tab + 8 * LS::TS);
    typename LS::ST *slots = (typename LS::ST *)(smem_raw + LanesTable<MAXD>::bytes);
    { // component table from the float blob in global memory: at pdf[0].foff, nc, then per
      // component: log-normalisation, m[fs], 1/s[fs] (fs = fstride >= ndim, zero-padded)
        const float *blob = p.fblob + p.pdf[0].foff;
        const int nc = (int)blob[0], fs = p.pdf[0].fstride, S = 1 + 2 * fs;
        for (int idx = threadIdx.x; idx < 8 * LS::TS; idx += blockDim.x) {
            const int cc = idx / LS::TS, j = idx % LS::TS, i = 2 * j;
            float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
            if (cc < nc && j < MAXD / 2) {
                const float *base = blob + 1 + cc * S;
                t = make_float4(i < fs ? base[1 + i] : 0.f, i < fs ? base[1 + fs + i] : 0.f,
                                i + 1 < fs ? base[2 + i] : 0.f, i + 1 < fs ? base[2 + fs + i] : 0.f);
            }
            tab[idx] = t;
        }
        for (int cc = threadIdx.x; cc < 8; cc += blockDim.x) { lcn[cc] = cc < nc ? blob[1 + cc * S] : 0.f; }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
    if (warp * LS::G >= p.nchains) { return; } // whole warps only: the shuffles name all 32 lanes
    LS s(p, fc, tab, lcn, slots, lane / LS::G, lane % LS::G, warp * LS::G + lane % LS::G);
    if (p.mode == KMODE_CALIB) { s.calibrate(p.nsteps); }
    else { s.run(p.nsteps, p.mode == KMODE_SAMPLE); }
    s.store_state();
}

// per-thread accumulator slots of a configuration: CPL per vector observable, 1 per scalar
template <int MAXD, int LPC>
size_t mcig_lanes_smem(const KParams &p, bool kahan)
{
    size_t ns = 0;
    for (int o = 0; o < p.nobs; ++o) {
        ns += (p.obs[o].kind == MCIG_OBS_XND || p.obs[o].kind == MCIG_OBS_X2) ? MAXD / LPC : 1;
    }
    return LanesTable<MAXD>::bytes + ns * MCIG_FAST_BLOCK * (kahan ? sizeof(float2) : sizeof(double));
}

template <int MAXD, int LPC, bool KAHAN, bool GAUSS>
void mcig_lanes_launch(const KParams &p0, const FastConst *fc, int /*movetype*/, int /*grid*/, int /*block*/,
                       size_t /*smem*/, cudaStream_t st)
{
    auto k = mcig_lanes_kernel<MAXD, LPC, KAHAN, GAUSS>;
    KParams p = p0;
    int ns = 0; // per-lane accumulator slot of each observable
    for (int o = 0; o < p.nobs; ++o) {
        p.obs[o].lslot = ns;
        ns += (p.obs[o].kind == MCIG_OBS_XND || p.obs[o].kind == MCIG_OBS_X2) ? MAXD / LPC : 1;
    }
    const size_t smem = mcig_lanes_smem<MAXD, LPC>(p, KAHAN);
    mcig_smem_attrs((const void *)k, smem);
    const int64_t threads = (int64_t)p.nchains * LPC;
    const int grid = (int)((threads + MCIG_FAST_BLOCK - 1) / MCIG_FAST_BLOCK);
    k<<<grid, MCIG_FAST_BLOCK, smem, st>>>(p, *fc);
}
