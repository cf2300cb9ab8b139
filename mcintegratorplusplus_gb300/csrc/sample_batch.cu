// Persistent batched sampling kernel: many independent integrals (each its own KParams:
// dimension, sampling functions, move, observables, seed) in ONE launch.  The warps pull
// work items from one atomic queue sorted longest-first over the whole batch; an item is
// up to 32 chains of integrals that share a code variant (chains of similar cost side by
// side, so small integrals share a warp instead of leaving its lanes idle), one chain per
// lane (`BatchLane`), and each lane runs the whole of MCI::integrate for its chain
// (findMRT2Step, burn-in, sampling with the accumulators; reference
// src/MCIntegrator.cpp:43-82).
//
// Two codes run in the same launch, chosen per item:
//  * the block-separable sampler (below) for the uneven-batch form: MultiStepMove of
//    single-coordinate sub-moves (src/MultiStepMove.cpp:6-47) whose sub-pdfs and sampling
//    functions are isotropic Gaussian factors over coordinate ranges, observables x.x per
//    block or in all.  The walker lives in shared memory (one column per lane, so a
//    sub-step's random coordinate is one conflict-free access), and the log densities and
//    the observables are kept as sums of squares over the ranges, updated by each accepted
//    sub-step, so an outer step costs O(sub-steps + ranges) instead of the O(ndim)
//    re-evaluation of the general sampler; the sums are recomputed exactly every 256 steps so
//    that float rounding cannot drift.  Its sub-step loop comes in three unrollings, which the
//    autotuner chooses per ndim bucket.
//  * the general float sampler (mcig_generic.cuh) for every other configuration, and the
//    general double sampler for FP64 batches (Philox or replayed draws), whose chains give
//    the numbers of their own integrate with the general kernel.
#include "mcig_generic.cuh"
#include "mcig_calib.cuh"
#include "mcig_batch.h"

// shared memory of the block-separable sampler, per lane: the walker (`walk` floats, the
// batch's largest ndim), the running sums (`nslot` slots: Kahan float2 or double) and the
// step's undo log (`nundo` sub-steps: coordinate index and old value), each [count][block]
struct BatchLayout {
    int walk, nslot, nundo;
    template <bool KAHAN> __host__ __device__ size_t bytes(int block) const
    {
        return (size_t)block * (walk * sizeof(float) + nslot * (KAHAN ? sizeof(float2) : sizeof(double)) +
                                nundo * (sizeof(int) + sizeof(float)));
    }
};

template <bool KAHAN, int UNR, bool GAUSS> // GAUSS: Gaussian (else uniform) sub-move draws
struct BlockSepSampler {
    using Slot = FastSlot<KAHAN>;
    using ST = typename Slot::T;
    static constexpr int MR = MCIG_BS_MAXR;
    const KParams &p;
    const BatchSep &b;
    const int c;
    float *xs;   // coordinate i of the walker at xs[i * ws]
    const int ws;
    ST *sl;      // running sum of value j at sl[j * ws]
    int *uidx;   // undo log of the step: sub-step j's coordinate and old value at [j * ws]
    float *uval;
    float st[MCIG_MAXTYPES];
    uint64_t ctr;
    uint32_t s0, s1;
    float S[MR]; // sums of x_i^2 over the ranges
    int since;

    __device__ BlockSepSampler(const KParams &pp, const BatchSep &bb, int cc, float *x0, int stride, ST *slots, int *ui,
                               float *uv)
        : p(pp), b(bb), c(cc), xs(x0), ws(stride), sl(slots), uidx(ui), uval(uv)
    {
        for (int i = 0; i < p.ndim; ++i) { xs[i * ws] = (float)p.x[(size_t)i * p.nchains + c]; }
#pragma unroll
        for (int t = 0; t < MCIG_MAXTYPES; ++t) { st[t] = t < p.ntypes ? (float)p.step[(size_t)t * p.nchains + c] : 0.f; }
        ctr = p.ctr[c];
        recompute();
    }

    __device__ __forceinline__ void recompute()
    {
#pragma unroll
        for (int r = 0; r < MR; ++r) {
            float s = 0.f;
            if (r < b.nr) {
                for (int i = b.ra[r]; i < b.rb[r]; ++i) {
                    const float v = xs[i * ws];
                    s = fmaf(v, v, s);
                }
            }
            S[r] = s;
        }
        since = 0;
    }

    __device__ __forceinline__ P4 block(uint32_t sub, uint32_t tag, uint32_t blk) const
    {
        return philox4x32_10(s0, s1, (uint32_t)c, (sub << 16) | (tag << 12) | blk, p.key0, p.key1);
    }

    // the draw of coordinate i in sub-step `sub`: move_draws<float> of block i / 4, entry i % 4
    __device__ __forceinline__ float draw1(uint32_t sub, int i) const
    {
        const P4 q = block(sub, TAG_MOVE, (uint32_t)(i >> 2));
        const int k = i & 3;
        if constexpr (GAUSS) {
            float z0, z1;
            box_muller_f(k < 2 ? q.a : q.c, k < 2 ? q.b : q.d, z0, z1);
            return (k & 1) ? z1 : z0;
        }
        const uint32_t w = k == 0 ? q.a : (k == 1 ? q.b : (k == 2 ? q.c : q.d));
        return u01_f(w) * 2.0f - 1.0f;
    }

    // MCI::doStepMRT2 with the MultiStepMove: a nested chain of single-coordinate moves on
    // the sub-pdfs, then the Metropolis test of its end point with pdfAcc * oldPDF/newPDF
    __device__ bool step()
    {
        s0 = (uint32_t)ctr;
        s1 = (uint32_t)(ctr >> 32);
        float dsub = 0.f; // log sub-density change of the sub-chain
        float dout = 0.f; // log change of the sampling functions
        int nu = 0;
        const int ns = p.ms_nsteps;
#pragma unroll UNR
        for (int s = 0; s < ns; ++s) {
            const uint32_t sub = 1 + s;
            const int i = (int)__umulhi(block(sub, TAG_INDEX, 0).a, (uint32_t)p.ndim);
            const float xi = xs[i * ws];
            const float xn = fmaf(st[0], draw1(sub, i), xi);
            const float diff = xn * xn - xi * xi;
            float dl = 0.f, dp = 0.f;
            bool in[MR];
#pragma unroll
            for (int r = 0; r < MR; ++r) {
                in[r] = r < b.nr && i >= b.ra[r] && i < b.rb[r];
                if (in[r]) {
                    dl = fmaf(-b.sc[r], diff, dl);
                    dp = fmaf(-b.pc[r], diff, dp);
                }
            }
            if (__log2f(accept_draw<float>(block(sub, TAG_ACCEPT, 0))) <= dl * 1.44269504f) {
                uidx[nu * ws] = i;
                uval[nu * ws] = xi;
                ++nu;
                xs[i * ws] = xn;
#pragma unroll
                for (int r = 0; r < MR; ++r) {
                    if (in[r]) { S[r] += diff; }
                }
                dsub += dl;
                dout += dp;
            }
        }
        // pdfAcc * oldPDF/newPDF of the sub-pdfs, in log
        const bool acc = __log2f(accept_draw<float>(block(0, TAG_ACCEPT, 0))) <= (dout - dsub) * 1.44269504f;
        if (!acc && nu > 0) { // back to the walker of the step's start, and its exact sums
            for (int j = nu - 1; j >= 0; --j) { xs[uidx[j * ws] * ws] = uval[j * ws]; }
            recompute();
        }
        ++ctr;
        if (++since >= 256) { recompute(); }
        return acc;
    }

    __device__ __forceinline__ void put(const ObsDesc &od, int j, uint32_t kk, bool flush, uint32_t blk, float v)
    {
        const size_t nc = (size_t)p.nchains;
        if (od.acc == MCIG_ACC_FULL) {
            const size_t row = (size_t)p.acc_offset + kk;
            if (od.full32) { ((float *)od.data)[(row * od.nv + j) * nc + c] = v; }
            else { ((double *)od.data)[(row * od.nv + j) * nc + c] = (double)v; }
            return;
        }
        ST &s = sl[(od.voff + j) * ws];
        Slot::add(s, v);
        if (od.acc == MCIG_ACC_BLOCK && flush) {
            ((double *)od.data)[((size_t)blk * od.nv + j) * nc + c] = Slot::get(s) * od.inv_bs;
            Slot::zero(s);
        }
    }

    // observable o after step r (AccumulatorInterface.cpp:31-60): x.x per block (X2BLOCK) or
    // in all (X2SUM), the range sums orng[o] ...
    __device__ __forceinline__ void obs_step(int o, const ObsDesc &od, uint32_t r)
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
        const int base = b.orng[o];
#pragma unroll
        for (int rr = 0; rr < MR; ++rr) {
            if (rr >= base && rr < base + od.nv) { put(od, rr - base, kk, flush, blk, S[rr]); }
        }
    }

    __device__ void run_sample(int64_t n)
    {
        for (int j = 0; j < p.nobsdim; ++j) { Slot::zero(sl[j * ws]); }
        uint32_t na = 0;
        for (uint32_t r = 0; r < (uint32_t)n; ++r) {
            na += step() ? 1u : 0u;
#pragma unroll
            for (int o = 0; o < MCIG_BS_MAXOBS; ++o) {
                if (o < p.nobs) { obs_step(o, p.obs[o], r); }
            }
        }
        for (int o = 0; o < p.nobs; ++o) { // SimpleAccumulator::_finalize
            const ObsDesc &od = p.obs[o];
            if (od.acc != MCIG_ACC_SIMPLE) { continue; }
            const double normf = 1. / (double)(1 + (n - 1) / od.nskip);
            for (int j = 0; j < od.nv; ++j) { ((double *)od.data)[(size_t)j * p.nchains + c] = Slot::get(sl[(od.voff + j) * ws]) * normf; }
        }
        p.nacc[c] = na;
        p.nrej[c] = n - na;
    }

    __device__ void run_steps(int64_t n)
    {
        int64_t na = 0;
        for (int64_t r = 0; r < n; ++r) { na += step() ? 1 : 0; }
        p.nacc[c] = na;
        p.nrej[c] = n - na;
    }

    // MCI::findMRT2Step (MCIntegrator.cpp:87-168) for this chain (FastSampler::calibrate's loop)
    __device__ void run_calibration(int64_t MIN_STAT)
    {
        int cons = 0, counter = 0;
        int64_t na = 0;
        while (calib_more(p, cons, counter)) {
            na = 0;
            for (int64_t r = 0; r < MIN_STAT; ++r) { na += step() ? 1 : 0; }
            calib_update(p, na, MIN_STAT, cons, st);
            ++counter;
        }
        p.nacc[c] = na;
        p.nrej[c] = (counter > 0) ? MIN_STAT - na : 0;
    }

    __device__ void store_state()
    {
        for (int i = 0; i < p.ndim; ++i) { p.x[(size_t)i * p.nchains + c] = (double)xs[i * ws]; }
        for (int t = 0; t < p.ntypes; ++t) { p.step[(size_t)t * p.nchains + c] = (double)st[t]; }
        p.ctr[c] = ctr;
    }
};

template <bool KAHAN, int UNR, bool GAUSS>
__device__ __noinline__ void batch_run_bs(const KParams &p, const BatchPhase &q, const BatchSep &b, int c, unsigned char *smem,
                                          BatchLayout lay)
{
    using BS = BlockSepSampler<KAHAN, UNR, GAUSS>;
    using ST = typename BS::ST;
    const size_t ws = blockDim.x;
    float *xs = (float *)smem + threadIdx.x;
    ST *sl = (ST *)(smem + ws * lay.walk * sizeof(float)) + threadIdx.x;
    int *ui = (int *)(smem + ws * (lay.walk * sizeof(float) + lay.nslot * sizeof(ST))) + threadIdx.x;
    float *uv = (float *)(smem + ws * (lay.walk * sizeof(float) + lay.nslot * sizeof(ST) + lay.nundo * sizeof(int))) + threadIdx.x;
    BS s(p, b, c, xs, (int)ws, sl, ui, uv);
    if (q.do_find) { s.run_calibration(q.min_stat); }
    if (q.ndecorr > 0) { s.run_steps(q.ndecorr); }
    s.run_sample(p.nsteps);
    s.store_state();
}

// at most 128 registers: the block-separable sampler runs without spills (at 85 registers it
// spilled 100-900 bytes per thread in its step loop), and 16 warps per SM still hold every task
// of a batch of ~64,000 chains at once (13 warps per SM); the general sampler keeps its walker
// arrays in local memory either way
template <class R, int RNG, bool KAHAN>
__global__ void __launch_bounds__(256, 2) mcig_batch_kernel(const KParams *__restrict__ cfg, const BatchPhase *__restrict__ ph,
                                                            const BatchSep *__restrict__ sep, const BatchTask *__restrict__ tasks,
                                                            const BatchLane *__restrict__ lanes, int ntasks, int *counter,
                                                            BatchLayout lay)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    while (true) {
        int t = 0;
        if (lane == 0) { t = atomicAdd(counter, 1); }
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= ntasks) { break; }
        const BatchTask task = tasks[t];
        if (lane >= task.count) { continue; }
        const BatchLane li = lanes[(size_t)t * 32 + lane]; // this lane's integral and chain
        const KParams &p = cfg[li.integral];
        const BatchPhase &q = ph[li.integral];
        const int c = li.chain;
        if constexpr (std::is_same<R, float>::value && RNG == RNG_PHILOX) {
            if (task.variant > 0) {
                const BatchSep &b = sep[li.integral];
                switch (task.variant) { // 1 + unroll index, + 3 for Gaussian sub-moves
                case 1: batch_run_bs<KAHAN, 1, false>(p, q, b, c, smem_raw, lay); break;
                case 2: batch_run_bs<KAHAN, 2, false>(p, q, b, c, smem_raw, lay); break;
                case 3: batch_run_bs<KAHAN, 4, false>(p, q, b, c, smem_raw, lay); break;
                case 4: batch_run_bs<KAHAN, 1, true>(p, q, b, c, smem_raw, lay); break;
                case 5: batch_run_bs<KAHAN, 2, true>(p, q, b, c, smem_raw, lay); break;
                default: batch_run_bs<KAHAN, 4, true>(p, q, b, c, smem_raw, lay); break;
                }
                continue;
            }
        }
        GenericSampler<R, RNG, KAHAN> s(p, c, p.fblob);
        if (q.do_find) { s.run_calibration(q.movetype, q.min_stat); }
        if (q.ndecorr > 0) { s.run_steps(q.movetype, q.ndecorr); }
        s.run_sample(q.movetype, p.nsteps);
        s.store_state();
    }
}

template <class R, int RNG, bool KAHAN>
static size_t smem_k(const BatchLayout &lay, int block)
{
    return std::is_same<R, float>::value ? lay.bytes<KAHAN>(block) : 0;
}

template <class R, int RNG, bool KAHAN>
static void launch_k(const KParams *cfg, const BatchPhase *ph, const BatchSep *sep, const BatchTask *tasks,
                     const BatchLane *lanes, int ntasks, int *counter, int grid, int block, const BatchLayout &lay,
                     cudaStream_t st)
{
    auto k = mcig_batch_kernel<R, RNG, KAHAN>;
    const size_t smem = smem_k<R, RNG, KAHAN>(lay, block);
    if (smem > 48 * 1024) { cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); }
    k<<<grid, block, smem, st>>>(cfg, ph, sep, tasks, lanes, ntasks, counter, lay);
}

template <class R, int RNG, bool KAHAN>
static int blocks_per_sm_k(const BatchLayout &lay, int block)
{
    auto k = mcig_batch_kernel<R, RNG, KAHAN>;
    const size_t smem = smem_k<R, RNG, KAHAN>(lay, block);
    if (smem > 48 * 1024) { cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); }
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, block, smem);
    return n;
}

void mcig_batch_launch(int prec, int rng, const KParams *cfg, const BatchPhase *ph, const BatchSep *sep,
                       const BatchTask *tasks, const BatchLane *lanes, int ntasks, int *counter, int grid, int block,
                       int walk, int nslot, int nundo, cudaStream_t st)
{
    const BatchLayout lay{walk, nslot, nundo};
    if (prec == MCIG_PREC_FP64) {
        if (rng == RNG_TAPE) { launch_k<double, RNG_TAPE, false>(cfg, ph, sep, tasks, lanes, ntasks, counter, grid, block, lay, st); }
        else { launch_k<double, RNG_PHILOX, false>(cfg, ph, sep, tasks, lanes, ntasks, counter, grid, block, lay, st); }
    } else if (prec == MCIG_PREC_FP32) {
        launch_k<float, RNG_PHILOX, true>(cfg, ph, sep, tasks, lanes, ntasks, counter, grid, block, lay, st);
    } else {
        launch_k<float, RNG_PHILOX, false>(cfg, ph, sep, tasks, lanes, ntasks, counter, grid, block, lay, st);
    }
}

int mcig_batch_blocks_per_sm(int prec, int rng, int block, int walk, int nslot, int nundo)
{
    const BatchLayout lay{walk, nslot, nundo};
    if (prec == MCIG_PREC_FP64) {
        return rng == RNG_TAPE ? blocks_per_sm_k<double, RNG_TAPE, false>(lay, block) : blocks_per_sm_k<double, RNG_PHILOX, false>(lay, block);
    }
    return prec == MCIG_PREC_FP32 ? blocks_per_sm_k<float, RNG_PHILOX, true>(lay, block) : blocks_per_sm_k<float, RNG_PHILOX, false>(lay, block);
}
