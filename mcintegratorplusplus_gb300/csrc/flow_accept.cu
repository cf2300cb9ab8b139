// Metropolis-Hastings test of the learned proposal (independence proposal x' = f(z)) for a
// single sampling function whose log density the register-resident kernel evaluates as
// straight-line code: exp(-x.x), a precision matrix or a mixture of at most 8 Gaussians,
// ndim <= 32.  One thread per chain, walker and proposal in registers (padded to MAXD with
// zeros), the sampling-function data as constant-bank operands (FastConst):
//   log u <= [log p(x') - log p(x)] + [log q(x) - log q(x')],
// then the Full accumulators record the observables at the chain's position (row krow).
// The general test in mcig_capi.cu (flow_accept_kernel) evaluates the sampling functions
// through the general kernel's runtime switch with the walker in local memory; both sides
// of the ratio use the same log density either way, so the target is unchanged.
#include "mcig_fast.cuh"
#include "mcig_generic.cuh"
#include "mcig_launchers.h"

template <int MAXD, int PK>
__global__ void __launch_bounds__(128) flow_accept_fast_kernel(const KParams p, const FastConst fc, const float *xprop,
                                                               const float *lq_prop, const float *lq_cur, uint64_t cycle,
                                                               int64_t krow, int64_t *nacc_flow)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= p.nchains) { return; }
    float x[MAXD], xp[MAXD];
#pragma unroll
    for (int i = 0; i < MAXD; ++i) { // both chain-minor; padding 0
        x[i] = i < p.ndim ? (float)p.x[(size_t)i * p.nchains + c] : 0.f;
        xp[i] = i < p.ndim ? xprop[(size_t)i * p.nchains + c] : 0.f;
    }
    float dl = lq_cur[c] - lq_prop[c];
    dl += fast_logp<MAXD, PK>(p, fc, xp) - fast_logp<MAXD, PK>(p, fc, x);
    const P4 q = philox4x32_10((uint32_t)cycle, (uint32_t)(cycle >> 32), (uint32_t)c, TAG_FLOW_ACCEPT << 12,
                               p.key0 ^ 0x6A09E667u, p.key1 ^ 0xBB67AE85u);
    const bool acc = isfinite(dl) && (__log2f(accept_draw<float>(q)) <= dl * 1.44269504f);
    if (acc) {
#pragma unroll
        for (int i = 0; i < MAXD; ++i) {
            x[i] = xp[i];
            if (i < p.ndim) { p.x[(size_t)i * p.nchains + c] = (double)xp[i]; }
        }
        nacc_flow[c] += 1;
    }
    if (krow < 0) { return; }
    float xo[MAXD]; // the observables index the walker at run time
#pragma unroll
    for (int i = 0; i < MAXD; ++i) { xo[i] = x[i]; }
    float vals[2 * MAXD + 8];
    for (int o = 0; o < p.nobs; ++o) {
        const ObsDesc &od = p.obs[o];
        obs_eval<float>(p, od, xo, vals, p.fblob);
        const size_t base = (size_t)krow * od.nv * p.nchains + c;
        for (int j = 0; j < od.nv; ++j) {
            if (od.full32) { ((float *)od.data)[base + (size_t)j * p.nchains] = vals[j]; }
            else { ((double *)od.data)[base + (size_t)j * p.nchains] = (double)vals[j]; }
        }
    }
}

template <int MAXD, int PK>
static void flow_accept_fast_launch(const KParams &p, const FastConst *fc, const float *xprop, const float *lq_prop,
                                    const float *lq_cur, uint64_t cycle, int64_t krow, int64_t *nacc_flow, cudaStream_t st)
{
    const int tb = 128, tg = (int)((p.nchains + tb - 1) / tb);
    flow_accept_fast_kernel<MAXD, PK><<<tg, tb, 0, st>>>(p, *fc, xprop, lq_prop, lq_cur, cycle, krow, nacc_flow);
}

mcig_flow_accept_fn mcig_flow_accept_launcher(int maxd, int pk)
{
#define MCIG_FA(M)                                                                                                      \
    switch (pk) {                                                                                                       \
    case PK_GAUSS: return flow_accept_fast_launch<M, PK_GAUSS>;                                                         \
    case PK_PREC: return flow_accept_fast_launch<M, PK_PREC>;                                                           \
    case PK_MIX: return flow_accept_fast_launch<M, PK_MIX>;                                                             \
    default: return nullptr;                                                                                            \
    }
    switch (maxd) {
    case 8: MCIG_FA(8)
    case 16: MCIG_FA(16)
    case 32: MCIG_FA(32)
    default: return nullptr;
    }
#undef MCIG_FA
}
