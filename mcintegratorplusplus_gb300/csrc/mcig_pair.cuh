// mcig_pair.cuh -- float sampling kernel with two lanes per chain for one precision-matrix
// or exp(-x.x) sampling function in 9..16 coordinates (the batched plain-Metropolis shape:
// 65,536 chains of a 16-D Gaussian with a dense precision matrix).
//
// The one-lane register-resident kernel (mcig_fast.cuh) needs ~124 registers per thread,
// so 65,536 chains are 12 warps per SM; with three warps per scheduler it issues in little
// more than half of the cycles, the rest being dependency latency (Philox rounds, the
// quadratic form's FMA chains, the MUFU of Box-Muller).  Here the two lanes of a chain
// share its step, so the same chains are twice the warps at two thirds of the registers:
//   * lane group l (lanes 16 l .. 16 l + 15, one chain each) owns coordinates [8 l, 8 l + 8),
//     i.e. the Philox move blocks 2 l and 2 l + 1 of the step, and draws and moves only those;
//   * the proposal's coordinates reach both lanes by shuffles as U x consumes them; lane
//     group l forms the rows 2 s + l (s = 0..7) of U x, each an FMA chain over ascending
//     columns from +0 (the one-lane kernel's order), the rows' coefficients read from a
//     shared-memory table in the order the chain consumes them (columns left of the
//     diagonal hold zeros, which leave the +0 start unchanged);
//   * both lanes square and sum the 16 row values in row order, and form x.x and the sum
//     of the coordinates over the gathered proposal in ascending order;
//   * on even steps r, lane group l draws the accept uniform of step r + l and a shuffle
//     hands it to the other group, so each step's accept block is formed once per chain.
// Log density, Metropolis decision, walker, Philox position and accumulator sums are the
// one-lane kernel's bit for bit (tests/test_pair.py).
// Lane layout: lane = 16 l + k holds chain 16 w + k of warp w, so each group's Full stores
// cover 16 consecutive chains (64 contiguous bytes).
#pragma once

#include "mcig_calib.cuh"

// first entry of column j in a lane group's coefficient table: column j feeds the slots
// 0 .. j / 2 (slot s forms row 2 s + l, whose columns start at 2 s), 72 entries in all
// (the sum over j' < j of j' / 2 + 1, in closed form)
__host__ __device__ __forceinline__ constexpr int pair_coef_off(int j)
{
    return (j % 2 == 0) ? (j / 2) * (j / 2 + 1) : (j / 2 + 1) * (j / 2 + 1);
}

// MOMENTS: every observable is x (XND) or x.x (X2SUM) with float Full data or a Simple/Block
// accumulator, so only those paths are compiled (FastSampler's MOMENTS); GAUSS: Gaussian
// (else uniform) move draws, known at compile time
template <int PK, bool KAHAN, bool MOMENTS = false, bool GAUSS = true>
struct PairSampler {
    static_assert(PK == PK_PREC || PK == PK_GAUSS, "the pair kernel serves one precision matrix or exp(-x.x)");
    static constexpr int MAXD = 16;            // coordinates (padded with zero steps)
    static constexpr int CPL = 8;              // coordinates per lane
    static constexpr int G = 16;               // chains per warp
    static constexpr int NCOEF = 72;           // coefficients per lane group
    static constexpr size_t TAB_BYTES = PK == PK_PREC ? 2 * NCOEF * sizeof(float) : 0;
    static constexpr unsigned FULL = 0xffffffffu;
    using Slot = FastSlot<KAHAN>;
    using ST = typename Slot::T;

    const KParams &p;
    const FastConst &fc;
    const float4 *tab;   // this lane group's 72 coefficients (18 float4)
    ST *slots;           // [nslot][MCIG_FAST_BLOCK]
    int l, k, c;         // coordinate group, chain in warp, chain
    bool valid;          // a chain of this launch
    float x[CPL], sto[CPL];
    float st[MCIG_MAXTYPES];
    float lp, xx, sx;    // log density, x.x and sum x_i of the walker
    float ua;            // accept uniform drawn on the last even step (step r + l)
    uint64_t ctr;
    bool need_xx, need_sx;

    __device__ static bool vec_kind(int kind) { return kind == MCIG_OBS_XND || kind == MCIG_OBS_X2; }

    __device__ PairSampler(const KParams &pp, const FastConst &ff, const float *tb, ST *sl, int lane_group,
                           int chain_in_warp, int chain)
        : p(pp), fc(ff), tab((const float4 *)tb), slots(sl), l(lane_group), k(chain_in_warp), c(chain)
    {
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
        ua = 1.f;
        need_xx = need_sx = false;
    }

    // x.x and the coordinate sum are formed with the log density only while observables
    // that read them are accumulated
    __device__ __forceinline__ void set_needs(bool sample)
    {
        need_xx = need_sx = false;
        for (int o = 0; o < p.nobs && sample; ++o) {
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

    // coefficient u of the lane group's table (compile-time u: the float4 loads are shared)
    __device__ __forceinline__ float coef(int u) const
    {
        const float4 v = tab[u >> 2];
        return (u & 3) == 0 ? v.x : (u & 3) == 1 ? v.y : (u & 3) == 2 ? v.z : v.w;
    }

    // fast_logp<16, PK> of the chain's vector whose own coordinates this lane holds in `own`,
    // same operation order, with x.x and the coordinate sum of the vector (i ascending)
    __device__ __forceinline__ float logp(const float (&own)[CPL], float &xxo, float &sxo) const
    {
        float t[8];
#pragma unroll
        for (int s = 0; s < 8; ++s) { t[s] = 0.f; }
        float xx2 = 0.f, sx2 = 0.f;
#pragma unroll
        for (int j = 0; j < MAXD; ++j) {
            // the coefficient loads of a column are issued with it: hoisting all 18 float4
            // loads would take 72 registers
            if (PK == PK_PREC && j % 2 == 0) { asm volatile("" ::: "memory"); }
            const float xj = __shfl_sync(FULL, own[j % CPL], (j / CPL) * G + k);
            if (PK == PK_GAUSS || need_xx) { xx2 = fmaf(xj, xj, xx2); }
            if (need_sx) { sx2 += xj; }
            if constexpr (PK == PK_PREC) {
#pragma unroll
                for (int s = 0; s <= j / 2; ++s) { t[s] = fmaf(coef(pair_coef_off(j) + s), xj, t[s]); }
            }
        }
        xxo = xx2;
        sxo = sx2;
        if constexpr (PK == PK_GAUSS) {
            return -xx2;
        } else {
            float q = 0.f;
#pragma unroll
            for (int i = 0; i < MAXD; ++i) { // row i was formed in slot i / 2 by lane group i % 2
                const float ti = __shfl_sync(FULL, t[i / 2], (i % 2) * G + k);
                q = fmaf(ti, ti, q);
            }
            return fast_lp_of_q(q);
        }
    }

    // one Metropolis step (MCI::doStepMRT2, MCIntegrator.cpp:326-360), the r-th of a run of
    // steps; upd false: the chain takes no part (its lanes still join the shuffles)
    __device__ __forceinline__ bool step(bool upd, uint32_t r)
    {
        const uint32_t s0 = (uint32_t)ctr, s1 = (uint32_t)(ctr >> 32);
        if ((r & 1u) == 0u) { // accept uniforms of steps r (group 0) and r + 1 (group 1)
            const uint64_t ca = ctr + (uint64_t)l;
            ua = accept_draw<float>(philox4x32_10_rk((uint32_t)ca, (uint32_t)(ca >> 32), (uint32_t)c, TAG_ACCEPT << 12, fc.rk));
        }
        const float u = __shfl_sync(FULL, ua, (int)(r & 1u) * G + k);
        constexpr bool gauss = GAUSS;
        float xn[CPL];
#pragma unroll
        for (int b = 0; b < CPL / 4; ++b) {
            float d[4];
            move_draws<float>(philox4x32_10_rk(s0, s1, (uint32_t)c, (TAG_MOVE << 12) | (uint32_t)(l * (CPL / 4) + b), fc.rk),
                              gauss, d);
#pragma unroll
            for (int i = 0; i < 4; ++i) { xn[4 * b + i] = fmaf(sto[4 * b + i], d[i], x[4 * b + i]); }
        }
        float xxn, sxn;
        const float lpn = logp(xn, xxn, sxn);
        const bool acc = fast_accept(u, lpn, lp);
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

    __device__ __forceinline__ ST &slot(int j) { return slots[j * MCIG_FAST_BLOCK + threadIdx.x]; }

    // AccumulatorInterface::accumulate of the values v[0..NV) of an observable at accumulation
    // kk: value m is value j0 + m of the observable (nv values); Full: one store per value,
    // 16 chains of a lane group contiguous; Simple/Block: the running sums in the lane's
    // slots from od.lslot, the block mean written at the block's last index.  Every value is
    // written without a predicate when the observable has all of them (FastSampler::put).
    template <int NV>
    __device__ __forceinline__ void put(const ObsDesc &od, int j0, uint32_t kk, bool flush, uint32_t blk, const float *v)
    {
        const uint32_t ncs = (uint32_t)p.nchains; // value stride; j * ncs < 2^32 for any device array
        const bool all = j0 + NV <= od.nv;
        if (od.acc == MCIG_ACC_FULL) {
            const size_t row = (size_t)p.acc_offset + kk;
            if (od.full32) {
                float *dst = (float *)od.data + (row * (size_t)od.nv + j0) * ncs + c;
#pragma unroll
                for (int m = 0; m < NV; ++m) {
                    if (all || j0 + m < od.nv) { dst[m * ncs] = v[m]; }
                }
            } else if constexpr (!MOMENTS) {
                double *dst = (double *)od.data + (row * (size_t)od.nv + j0) * ncs + c;
#pragma unroll
                for (int m = 0; m < NV; ++m) {
                    if (all || j0 + m < od.nv) { dst[m * ncs] = (double)v[m]; }
                }
            }
            return;
        }
        ST *sl = slots + od.lslot * MCIG_FAST_BLOCK + threadIdx.x;
#pragma unroll
        for (int m = 0; m < NV; ++m) {
            if (all || j0 + m < od.nv) { Slot::add(sl[m * MCIG_FAST_BLOCK], v[m]); }
        }
        if (od.acc == MCIG_ACC_BLOCK && flush) {
            double *dst = (double *)od.data + ((size_t)blk * od.nv + j0) * ncs + c;
#pragma unroll
            for (int m = 0; m < NV; ++m) {
                if (all || j0 + m < od.nv) {
                    dst[m * ncs] = Slot::get(sl[m * MCIG_FAST_BLOCK]) * od.inv_bs;
                    Slot::zero(sl[m * MCIG_FAST_BLOCK]);
                }
            }
        }
    }

    // observableFunction of the built-in kinds (FastSampler::observe_put's values)
    __device__ __forceinline__ void observe(const ObsDesc &od, uint32_t kk, bool flush, uint32_t blk)
    {
        const int kind = od.kind;
        if constexpr (MOMENTS) {
            if (kind == MCIG_OBS_XND) {
                if (valid) { put<CPL>(od, l * CPL, kk, flush, blk, x); }
            } else if (valid && l == 0) {
                put<1>(od, 0, kk, flush, blk, &xx);
            }
            return;
        }
        if (vec_kind(kind)) {
            float v[CPL];
#pragma unroll
            for (int m = 0; m < CPL; ++m) { v[m] = kind == MCIG_OBS_XND ? x[m] : x[m] * x[m]; }
            if (valid) { put<CPL>(od, l * CPL, kk, flush, blk, v); }
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
        if (valid && l == 0) { put<1>(od, 0, kk, flush, blk, &v); }
    }

    // observable od after step r: accumulation index kk = r / nskip when nskip divides r
    // (AccumulatorInterface.cpp:31-60), block end when blocksize divides kk + 1
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

    // n < 2^32 steps (checked on the host); p.r0 is the global index of the first step
    // (chunked sampling)
    __device__ __forceinline__ void run(int64_t n, bool sample)
    {
        set_needs(sample);
        refresh();
        int nslot = 0;
        for (int o = 0; o < p.nobs; ++o) { nslot += vec_kind(p.obs[o].kind) ? CPL : 1; }
        for (int j = 0; j < nslot && sample; ++j) { Slot::zero(slot(j)); }
        const uint32_t n32 = (uint32_t)n;
        const uint32_t r0 = (uint32_t)p.r0;
        uint32_t na = 0;
        for (uint32_t r = 0; r < n32; ++r) {
            na += step(valid, r) ? 1u : 0u;
            if (!sample) { continue; }
#pragma unroll
            for (int o = 0; o < MCIG_FAST_UNROLLED_OBS; ++o) {
                if (o < p.nobs) { obs_step(p.obs[o], r0 + r); }
            }
            for (int o = MCIG_FAST_UNROLLED_OBS; o < p.nobs; ++o) { obs_step(p.obs[o], r0 + r); }
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
            if (p.acc_counts) {
                p.nacc[c] += na;
                p.nrej[c] += n - na;
            } else {
                p.nacc[c] = na;
                p.nrej[c] = n - na;
            }
        }
    }

    // MCI::findMRT2Step (MCIntegrator.cpp:87-168) for every chain of the warp, each on its
    // own (FastSampler::calibrate's loop); the warp runs until its last chain has finished
    __device__ __forceinline__ void calibrate(int64_t MIN_STAT)
    {
        int cons = 0, counter = 0;
        int64_t na = 0;
        set_needs(false);
        bool runc = valid && calib_more(p, cons, counter);
        while (__any_sync(FULL, runc)) {
            {
                float xx0, sx0;
                const float l0 = logp(x, xx0, sx0);
                if (runc) { lp = l0; }
            }
            int64_t nacc = 0;
            for (uint32_t r = 0; r < (uint32_t)MIN_STAT; ++r) { nacc += step(runc, r) ? 1 : 0; }
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

// 64 threads (two warps, 32 chains) per block; at most 80 registers per thread (no spills)
// keep 12 blocks on an SM: the chain counts the kernel serves by default (at most 32,768, 6.7
// blocks per SM) run in one wave
template <int PK, bool KAHAN, bool MOMENTS, bool GAUSS>
__global__ void __launch_bounds__(MCIG_FAST_BLOCK, 12) mcig_pair_kernel(const KParams p, const FastConst fc)
{
    using PS = PairSampler<PK, KAHAN, MOMENTS, GAUSS>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *tab = (float *)smem_raw; // [2][72]: lane group l's coefficients, column-major
    typename PS::ST *slots = (typename PS::ST *)(smem_raw + PS::TAB_BYTES);
    if constexpr (PK == PK_PREC) { // entry (j, s) of group l: U[2 s + l][j], 0 left of the diagonal
        for (int idx = threadIdx.x; idx < 2 * PS::NCOEF; idx += blockDim.x) {
            const int lg = idx / PS::NCOEF, u = idx % PS::NCOEF;
            int j = 0;
            while (j < 15 && pair_coef_off(j + 1) <= u) { ++j; }
            const int row = 2 * (u - pair_coef_off(j)) + lg;
            tab[idx] = (j >= row) ? fc.fconst[row * PS::MAXD + j] : 0.f;
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
    if (warp * PS::G >= p.nchains) { return; } // whole warps only: the shuffles name all 32 lanes
    const int lg = lane / PS::G;
    PS s(p, fc, tab + lg * PS::NCOEF, slots, lg, lane % PS::G, warp * PS::G + lane % PS::G);
    if (p.mode == KMODE_CALIB) { s.calibrate(p.nsteps); }
    else { s.run(p.nsteps, p.mode == KMODE_SAMPLE); }
    s.store_state();
}

template <int PK, bool KAHAN, bool MOMENTS, bool GAUSS>
void mcig_pair_launch(const KParams &p0, const FastConst *fc, int /*movetype*/, int /*grid*/, int /*block*/,
                      size_t /*smem*/, cudaStream_t st)
{
    using PS = PairSampler<PK, KAHAN, MOMENTS, GAUSS>;
    auto k = mcig_pair_kernel<PK, KAHAN, MOMENTS, GAUSS>;
    KParams p = p0;
    int ns = 0; // per-lane accumulator slot of each observable
    for (int o = 0; o < p.nobs; ++o) {
        p.obs[o].lslot = ns;
        ns += (p.obs[o].kind == MCIG_OBS_XND || p.obs[o].kind == MCIG_OBS_X2) ? PS::CPL : 1;
    }
    const size_t smem = PS::TAB_BYTES + (size_t)ns * MCIG_FAST_BLOCK * sizeof(typename PS::ST);
    mcig_smem_attrs((const void *)k, smem);
    const int64_t threads = (int64_t)p.nchains * 2;
    const int grid = (int)((threads + MCIG_FAST_BLOCK - 1) / MCIG_FAST_BLOCK);
    k<<<grid, MCIG_FAST_BLOCK, smem, st>>>(p, *fc);
}
