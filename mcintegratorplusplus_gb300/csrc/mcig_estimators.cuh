// mcig_estimators.cuh -- estimator kernels (reference src/Estimators.cpp, src/MJBlocker.cpp).
//
// One thread per series.  The input is an accumulator array laid out
// [n][nv][nchains] (chain-minor, so consecutive threads read consecutive
// addresses); series s = j * nchains + c is component j of chain c.  Results go
// to avg/err[c * ldo + off + j].  Arithmetic is double in the reference's
// operation order (compile with -fmad=false), so that on identical arrays the
// results equal the reference's to the last bit, up to the square root and
// division, which are correctly rounded on both sides.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

struct EstArgs {
    const void *data;   // [n][nv][nchains]
    int is_float;       // data element type: float (1) or double (0)
    int64_t n;          // samples per series
    int nv;             // components
    int nchains;
    double *avg, *err;  // outputs [nchains][ldo]
    int ldo, off;
    double *scratch;    // MJBlocker: [n][nv*nchains] doubles
    int one_d;          // 1-D estimator rounding (reference wrappers send ndim == 1 there)
};

__device__ __forceinline__ double est_load(const EstArgs &a, int64_t i, int64_t s)
{
    const int64_t idx = i * (int64_t)a.nv * a.nchains + s;
    return a.is_float ? (double)((const float *)a.data)[idx] : ((const double *)a.data)[idx];
}

__device__ __forceinline__ void est_store(const EstArgs &a, int64_t s, double av, double er)
{
    const int c = (int)(s % a.nchains), j = (int)(s / a.nchains);
    a.avg[(size_t)c * a.ldo + a.off + j] = av;
    a.err[(size_t)c * a.ldo + a.off + j] = er;
}

// OneDimUncorrelatedEstimator (:36-56) / MultiDimUncorrelatedEstimator (:125-155) on the
// values v(i), i < n, produced by the functor.
template <class F>
__device__ __forceinline__ void uncorr_core(int64_t n, F v, int one_d, double &average, double &error)
{
    const double SMALLEST_ERROR = 1.e-300;
    double s = 0., q = 0.;
    for (int64_t i = 0; i < n; ++i) {
        const double x = v(i);
        s = s + x;
        q = q + x * x;
    }
    const double norm = 1. / n;
    average = s * norm;
    double e = q * norm - average * average;
    if (one_d) { e = (e > SMALLEST_ERROR) ? sqrt(e / (n - 1.)) : 0.; }
    else { e = (e > SMALLEST_ERROR) ? sqrt(e * (1. / (n - 1.))) : 0.; }
    error = e;
}

// Kahan-compensated float sums of x (s1, c1) and x^2 (s2, c2); explicit round-to-nearest
// operations, so no kernel contracts x * x - c2 into an FMA differently from another
__device__ __forceinline__ void kahan2(float &s1, float &c1, float &s2, float &c2, float x)
{
    float y = __fsub_rn(x, c1), t = __fadd_rn(s1, y);
    c1 = __fsub_rn(__fsub_rn(t, s1), y);
    s1 = t;
    y = __fsub_rn(__fmul_rn(x, x), c2);
    t = __fadd_rn(s2, y);
    c2 = __fsub_rn(__fsub_rn(t, s2), y);
    s2 = t;
}

// Uncorrelated estimator on float samples (float precision modes): Kahan-compensated
// float sums of x and x^2 (four float operations per value instead of two
// double ones), combined in double with the reference's formula.
static __global__ void est_uncorr_f32_kernel(EstArgs a)
{
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= (int64_t)a.nv * a.nchains) { return; }
    const float *d = (const float *)a.data + s;
    const int64_t stride = (int64_t)a.nv * a.nchains;
    float s1 = 0.f, c1 = 0.f, s2 = 0.f, c2 = 0.f;
    auto add = [&](float x) { kahan2(s1, c1, s2, c2, x); };
    // 32 loads in flight per thread, then the sums in sample order: with one value per
    // series (65,536 series) one load at a time kept too few bytes in flight for HBM
    int64_t i = 0;
    for (; i + 32 <= a.n; i += 32) {
        float x[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) { x[k] = d[(i + k) * stride]; }
#pragma unroll
        for (int k = 0; k < 32; ++k) { add(x[k]); }
    }
    for (; i < a.n; ++i) { add(d[i * stride]); }
    const double SMALLEST_ERROR = 1.e-300;
    const double norm = 1. / a.n;
    const double average = ((double)s1 - (double)c1) * norm;
    double e = ((double)s2 - (double)c2) * norm - average * average;
    if (a.one_d) { e = (e > SMALLEST_ERROR) ? sqrt(e / (a.n - 1.)) : 0.; }
    else { e = (e > SMALLEST_ERROR) ? sqrt(e * (1. / (a.n - 1.))) : 0.; }
    est_store(a, s, average, e);
}

// The same estimator over rows [i0, i1) of the data, for sampling that runs in chunks:
// the Kahan sums of each series continue from `state` (zero for i0 == 0) and are saved
// there, and the chunk that ends at row a.n forms the result.  Every series sees the add
// sequence of est_uncorr_f32_kernel, so the result is that kernel's bit for bit.  A small
// grid strides over the series: the kernel runs beside the next chunk's sampling launch
// and reads the finished rows while the sampling kernel is bound by instruction issue.
static __global__ void est_uncorr_f32_chunk_kernel(EstArgs a, int64_t i0, int64_t i1, float4 *state)
{
    const int64_t S = (int64_t)a.nv * a.nchains;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < S; s += (int64_t)gridDim.x * blockDim.x) {
        const float *d = (const float *)a.data + s;
        float4 st = i0 > 0 ? state[s] : make_float4(0.f, 0.f, 0.f, 0.f);
        float s1 = st.x, c1 = st.y, s2 = st.z, c2 = st.w;
        auto add = [&](float x) { kahan2(s1, c1, s2, c2, x); };
        int64_t i = i0;
        for (; i + 32 <= i1; i += 32) {
            float x[32];
#pragma unroll
            for (int k = 0; k < 32; ++k) { x[k] = d[(i + k) * S]; }
#pragma unroll
            for (int k = 0; k < 32; ++k) { add(x[k]); }
        }
        for (; i < i1; ++i) { add(d[i * S]); }
        if (i1 < a.n) {
            state[s] = make_float4(s1, c1, s2, c2);
            continue;
        }
        const double SMALLEST_ERROR = 1.e-300;
        const double norm = 1. / a.n;
        const double average = ((double)s1 - (double)c1) * norm;
        double e = ((double)s2 - (double)c2) * norm - average * average;
        if (a.one_d) { e = (e > SMALLEST_ERROR) ? sqrt(e / (a.n - 1.)) : 0.; }
        else { e = (e > SMALLEST_ERROR) ? sqrt(e * (1. / (a.n - 1.))) : 0.; }
        est_store(a, s, average, e);
    }
}

static __global__ void est_noop_kernel(EstArgs a)
{ // NoopEstimator (:289-293): the first row is the result
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= (int64_t)a.nv * a.nchains) { return; }
    est_store(a, s, est_load(a, 0, s), 0.);
}

static __global__ void est_uncorr_kernel(EstArgs a)
{
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= (int64_t)a.nv * a.nchains) { return; }
    double av, er;
    uncorr_core(a.n, [&](int64_t i) { return est_load(a, i, s); }, a.one_d, av, er);
    est_store(a, s, av, er);
}

// calcErrDelta (Estimators.cpp:9-31)
__device__ __forceinline__ double fc_delta(int mode, const double *e)
{
    const int im = 4;
    switch (mode) {
    case 1: return (-0.5 * e[im - 1] + 0.5 * e[im + 1]);
    case 2: return ((1. / 12.) * e[im - 2] - (2. / 3.) * e[im - 1] + (2. / 3.) * e[im + 1] - (1. / 12.) * e[im + 2]);
    case 3: return (-(1. / 60.) * e[im - 3] + (3. / 20.) * e[im - 2] - 0.75 * e[im - 1] + 0.75 * e[im + 1]
                    - (3. / 20.) * e[im + 2] + (1. / 60.) * e[im + 3]);
    case 4: return ((1. / 280.) * e[im - 4] - (4. / 105.) * e[im - 3] + 0.2 * e[im - 2] - 0.8 * e[im - 1]
                    + 0.8 * e[im + 1] - 0.2 * e[im + 2] + (4. / 105.) * e[im + 3] - (1. / 280.) * e[im + 4]);
    default: return 0.;
    }
}

// FCBlockerEstimator (Estimators.cpp:82-122 / 191-246): block estimators for 6..50
// blocks, plateau of the finite-difference slope of the error.
static __global__ void est_fc_kernel(EstArgs a)
{
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= (int64_t)a.nv * a.nchains) { return; }
    constexpr int MIN_BLOCKS = 6, MAX_BLOCKS = 50, MAX_PLATEAU_AVERAGE = 4;
    constexpr int NAV = MAX_BLOCKS - MIN_BLOCKS + 1;
    double av[NAV], er[NAV];
    for (int i1 = 0; i1 < NAV; ++i1) {
        const int nb = i1 + MIN_BLOCKS;
        const int64_t nper = a.n / nb;
        const double norm = 1. / nper;
        // block means, then the uncorrelated estimator over them (OneDim/MultiDimBlockEstimator)
        uncorr_core(
            nb,
            [&](int64_t b) {
                double t = 0.;
                for (int64_t i = b * nper; i < (b + 1) * nper; ++i) { t = t + est_load(a, i, s); }
                return t * norm;
            },
            a.one_d, av[i1], er[i1]);
    }
    constexpr int NACCD = NAV - 2 * MAX_PLATEAU_AVERAGE;
    double acc[NACCD];
    for (int i = 0; i < NACCD; ++i) { acc[i] = 0.; }
    for (int i2 = MAX_PLATEAU_AVERAGE; i2 < NACCD + MAX_PLATEAU_AVERAGE; ++i2) {
        for (int i1 = 1; i1 <= MAX_PLATEAU_AVERAGE; ++i1) {
            acc[i2 - MAX_PLATEAU_AVERAGE] = acc[i2 - MAX_PLATEAU_AVERAGE] + fc_delta(i1, er + i2 - 4);
        }
    }
    int imin = 0;
    for (int i2 = 1; i2 < NACCD; ++i2) {
        if (fabs(acc[i2]) < fabs(acc[imin])) { imin = i2; }
    }
    const int k = imin + MAX_PLATEAU_AVERAGE;
    est_store(a, s, 0.2 * (av[k - 2] + av[k - 1] + av[k] + av[k + 1] + av[k + 2]),
              0.2 * (er[k - 2] + er[k - 1] + er[k] + er[k + 1] + er[k + 2]));
}

// chi^2 0.95 quantiles, k + 1 degrees of freedom (MJBlocker.cpp:6-13)
static __constant__ double c_mj_quantile[64] = {
    3.841459, 5.991465, 7.814728, 9.487729, 11.070498, 12.591587, 14.067140, 15.507313,
    16.918978, 18.307038, 19.675138, 21.026070, 22.362032, 23.684791, 24.995790, 26.296228,
    27.587112, 28.869299, 30.143527, 31.410433, 32.670573, 33.924438, 35.172462, 36.415029,
    37.652484, 38.885139, 40.113272, 41.337138, 42.556968, 43.772972, 44.985343, 46.194260,
    47.399884, 48.602367, 49.801850, 50.998460, 52.192320, 53.383541, 54.572228, 55.758479,
    56.942387, 58.124038, 59.303512, 60.480887, 61.656233, 62.829620, 64.001112, 65.170769,
    66.338649, 67.504807, 68.669294, 69.832160, 70.993453, 72.153216, 73.311493, 74.468324,
    75.623748, 76.777803, 77.930524, 79.081944, 80.232098, 81.381015, 82.528727, 83.675261};

// MJBlocker::estimate (MJBlocker.cpp:127-154).  The blocking transform runs in
// place on a double copy of the series in scratch ([n][S], S = nv*nchains);
// X = x - mean is formed on the fly exactly as the reference stores it
// (:58-65, :100).  When no level passes the test (constant data) the last
// level is used, where the reference would read one level past its arrays.
static __global__ void est_mj_kernel(EstArgs a)
{
    const int64_t S = (int64_t)a.nv * a.nchains;
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= S) { return; }
    double *x = a.scratch + s;
    int npow = 0;
    while ((1LL << npow) < a.n) { ++npow; }
    double mean = 0.;
    for (int64_t i = 0; i < a.n; ++i) {
        const double v = est_load(a, i, s);
        x[i * S] = v;
        mean = mean + v;
    }
    mean = mean / a.n;
    double var[64], gam[64];
    int64_t nred = a.n;
    for (int k = 0; k < npow; ++k) {
        double v = 0., g = 0.;
        double Xprev = x[0] - mean;
        v = v + Xprev * Xprev;
        for (int64_t i = 1; i < nred; ++i) {
            const double X = x[i * S] - mean;
            v = v + X * X;
            g = g + Xprev * X;
            Xprev = X;
        }
        var[k] = v / nred;
        gam[k] = g / nred;
        for (int64_t i = 0; i < nred / 2; ++i) { x[i * S] = 0.5 * (x[(2 * i) * S] + x[(2 * i + 1) * S]); }
        nred = nred / 2;
    }
    // M_k (reversed) and cumulative sums (:106-123)
    double M[64], Ms[64];
    for (int i = 0; i < npow; ++i) {
        const double r = gam[i] / var[i];
        M[npow - i - 1] = (r * r) * ldexp(1.0, npow - i);
    }
    for (int i = 0; i < npow; ++i) {
        double t = 0.;
        for (int j = 0; j <= i; ++j) { t = t + M[j]; }
        Ms[i] = t;
    }
    int k;
    for (k = npow - 1; k >= 0; --k) {
        if (Ms[k] < c_mj_quantile[k]) { break; }
    }
    k = npow - (k + 1);
    if (k > npow - 1) { k = npow - 1; }
    if (k < 0) { k = 0; }
    est_store(a, s, mean, npow > 0 ? sqrt(var[k] / ldexp(1.0, npow - k)) : 0.);
}
