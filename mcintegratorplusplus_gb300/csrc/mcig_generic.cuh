// mcig_generic.cuh -- the general sampling kernel: every move, sampling function,
// observable, accumulator and domain of the device path, with runtime loops over
// the coordinates (walker arrays in thread-local memory, ndim <= MCIG_MAXDIM).
//
//   R = double: the reference's arithmetic and operation order.  The
//     translation unit is compiled with -fmad=false, so no product is fused
//     into an add (the reference is built for baseline x86-64, without FMA).
//     With RNG_TAPE the kernel consumes the reference's recorded draws and
//     reproduces its accept/reject sequence bit for bit.
//   R = float: float walker, log-space Metropolis test; sums of the
//     accumulators in float with Kahan compensation (KAHAN) or in double.
//
// The register-resident kernel for the common float configurations is in
// mcig_fast.cuh; this one serves everything else.
#pragma once

#include "mcig_common.cuh"
#include "mcig_plugin.cuh"

template <class R>
__device__ __forceinline__ R step_of_rt(const KParams &p, const R *st, int i)
{
    int t = 0;
    while (t + 1 < p.ntypes && i >= p.typeEnds[t]) { ++t; }
    return st[t];
}

template <class R>
__device__ __forceinline__ void periodic_wrap(R &v, double lb, double ub)
{
    // OrthoPeriodicDomain::applyDomain (OrthoPeriodicDomain.cpp:38-61).  The
    // loops are bounded; a coordinate still outside after that is clamped.
    const R L = (R)(ub - lb);
    int n = 0;
    while (v < (R)lb && n < MCIG_PERIODIC_MAXWRAP) { v += L; ++n; }
    while (v > (R)ub && n < MCIG_PERIODIC_MAXWRAP) { v -= L; ++n; }
    if (n >= MCIG_PERIODIC_MAXWRAP) { v = v < (R)lb ? (R)lb : (v > (R)ub ? (R)ub : v); }
}

// ------------------------------------------------------------------------
// sampling functions, double (test/common/TestMCIFunctions.hpp arithmetic;
// the same formulas as the oracle's pdf_* functions)
// ------------------------------------------------------------------------
__device__ __forceinline__ double proto_i_d(int kind, double v) { return kind == MCIG_PDF_GAUSS ? v * v : fabs(v); }

// the single proto value of the scalar-proto kinds (GAUSS_SUM, GAUSS_PREC, GAUSS_BLOCK, GAUSS_MIX)
static __device__ double pdf_proto_scalar_d(const KParams &p, const PdfDesc &d, const double *x)
{
    const int nd = p.ndim;
    switch (d.kind) {
    case MCIG_PDF_GAUSS_SUM: { // ThreeDimGaussianPDF::protoFunction (:134-137), any ndim
        double s = x[0] * x[0];
        for (int i = 1; i < nd; ++i) { s = s + x[i] * x[i]; }
        return s;
    }
    case MCIG_PDF_GAUSS_PREC: {
        const double *P = p.params + d.poff;
        double q = 0.;
        for (int i = 0; i < nd; ++i) {
            double t = 0.;
            for (int j = 0; j < nd; ++j) { t = t + P[i * nd + j] * x[j]; }
            q = q + x[i] * t;
        }
        return 0.5 * q;
    }
    case MCIG_PDF_GAUSS_BLOCK: {
        double s = 0.;
        for (int i = d.b0; i < d.b1; ++i) { s = s + x[i] * x[i]; }
        return s * d.c;
    }
    case MCIG_PDF_GAUSS_MIX: {
        const double *pp = p.params + d.poff;
        const int nc = (int)pp[0];
        const double *m = pp + 1 + nc, *sg = pp + 1 + nc + nc * nd, *lc = pp + 1 + nc + 2 * nc * nd;
        double e[16];
        double mx = -INFINITY;
        for (int c = 0; c < nc; ++c) {
            double a = lc[c];
            for (int i = 0; i < nd; ++i) {
                const double z = (x[i] - m[c * nd + i]) / sg[c * nd + i];
                a += -0.5 * (z * z);
            }
            e[c] = a;
            mx = a > mx ? a : mx;
        }
        double sum = 0.;
        for (int c = 0; c < nc; ++c) { sum += exp(e[c] - mx); }
        return -(mx + log(sum));
    }
    default: return 0.;
    }
}

// SamplingFunctionInterface::computeAcceptance (SamplingFunctionInterface.hpp:49-57).
// xo: accepted position, xn: proposal, partial: nchanged < ndim with the changed
// indices [lo, hi), po: cached scalar proto of xo, pn: scalar proto of xn (out).
static __device__ double pdf_accept_d(const KParams &p, const PdfDesc &d, const double *xo, const double *xn, bool partial,
                               int lo, int hi, double po, double &pn)
{
    const int nd = p.ndim;
    if (d.kind == MCIG_PDF_GAUSS || d.kind == MCIG_PDF_EXP) {
        if (partial) { // Gauss::updatedAcceptance (:181-189), ExpNDPDF::updatedAcceptance (:246-255)
            double e = 0.;
            for (int i = lo; i < hi; ++i) { e = e + (proto_i_d(d.kind, xn[i]) - proto_i_d(d.kind, xo[i])); }
            return exp(-e);
        }
        double e = 0.; // Gauss::acceptanceFunction (:174-179)
        for (int i = 0; i < nd; ++i) { e = e + proto_i_d(d.kind, xo[i]); }
        double f = 0.;
        for (int i = 0; i < nd; ++i) { f = f + proto_i_d(d.kind, xn[i]); }
        e = e - f;
        return exp(e);
    }
    pn = pdf_proto_scalar_d(p, d, xn);
    return exp(-pn + po); // ThreeDimGaussianPDF::acceptanceFunction (:144-147)
}

// samplingFunction at the stored protos of x (SamplingFunctionContainer::getOldSamplingFunction)
static __device__ double pdf_value_d(const KParams &p, const PdfDesc &d, const double *x, double po)
{
    if (d.kind == MCIG_PDF_GAUSS || d.kind == MCIG_PDF_EXP) {
        double s = 0.;
        for (int i = 0; i < p.ndim; ++i) { s = s + proto_i_d(d.kind, x[i]); }
        return exp(-s);
    }
    return exp(-po);
}

// ------------------------------------------------------------------------
// sampling functions, float (log density; parameter blob in shared memory)
//   GAUSS_PREC : U[ndim][fstride], upper Cholesky factor of P (x^T P x = |U x|^2)
//   GAUSS_MIX  : nc, then per component: log-normalisation, m[fstride], 1/s[fstride]
// ------------------------------------------------------------------------
static __device__ float pdf_logp_f(const KParams &p, const PdfDesc &d, const float *x, const float *blob)
{
    const int nd = p.ndim;
    switch (d.kind) {
    case MCIG_PDF_GAUSS_SUM:
    case MCIG_PDF_GAUSS: {
        float s = 0.f;
        for (int i = 0; i < nd; ++i) { s = fmaf(x[i], x[i], s); }
        return -s;
    }
    case MCIG_PDF_EXP: {
        float s = 0.f;
        for (int i = 0; i < nd; ++i) { s += fabsf(x[i]); }
        return -s;
    }
    case MCIG_PDF_GAUSS_PREC: {
        const float *U = blob + d.foff;
        float q = 0.f;
        for (int i = 0; i < nd; ++i) {
            float t = 0.f;
            for (int j = i; j < nd; ++j) { t = fmaf(U[i * d.fstride + j], x[j], t); }
            q = fmaf(t, t, q);
        }
        return -0.5f * q;
    }
    case MCIG_PDF_GAUSS_BLOCK: {
        float s = 0.f;
        for (int i = d.b0; i < d.b1; ++i) { s = fmaf(x[i], x[i], s); }
        return -(float)d.c * s;
    }
    case MCIG_PDF_GAUSS_MIX: {
        const float *b = blob + d.foff;
        const int nc = (int)b[0];
        const int stride = 1 + 2 * d.fstride;
        float e[16];
        float mx = -INFINITY;
        for (int c = 0; c < nc; ++c) {
            const float *cb = b + 1 + c * stride;
            float a = 0.f;
            for (int i = 0; i < nd; ++i) {
                const float z = (x[i] - cb[1 + i]) * cb[1 + d.fstride + i];
                a = fmaf(z, z, a);
            }
            a = fmaf(-0.5f, a, cb[0]);
            e[c] = a;
            mx = fmaxf(mx, a);
        }
        float sum = 0.f;
        for (int c = 0; c < nc; ++c) { sum += __expf(e[c] - mx); }
        return mx + __logf(sum);
    }
    default: return 0.f;
    }
}

// log p(xn) - log p(w) of a separable float sampling function when xn and w differ only
// in [lo, hi) (the float counterpart of the updatedAcceptance of Gauss / ExpNDPDF,
// TestMCIFunctions.hpp:181-189, :246-255); returns false for the other kinds
static __device__ bool pdf_delta_f(const PdfDesc &d, const float *w, const float *xn, int lo, int hi, float &delta)
{
    float s = 0.f;
    switch (d.kind) {
    case MCIG_PDF_GAUSS_SUM:
    case MCIG_PDF_GAUSS:
        for (int i = lo; i < hi; ++i) { s += xn[i] * xn[i] - w[i] * w[i]; }
        delta = -s;
        return true;
    case MCIG_PDF_EXP:
        for (int i = lo; i < hi; ++i) { s += fabsf(xn[i]) - fabsf(w[i]); }
        delta = -s;
        return true;
    case MCIG_PDF_GAUSS_BLOCK: {
        const int a = max(lo, d.b0), b = min(hi, d.b1);
        for (int i = a; i < b; ++i) { s += xn[i] * xn[i] - w[i] * w[i]; }
        delta = -(float)d.c * s;
        return true;
    }
    default: return false;
    }
}

// ------------------------------------------------------------------------
// observables (observableFunction of the test classes; oracle obs_eval)
// ------------------------------------------------------------------------
// log of the product of the sampling functions at x: double -sum_k (proto_k summed in
// index order), as the oracle; float sum_k log p_k (the float path's log densities)
static __device__ double logpdf_d(const KParams &p, const double *x)
{
    double s = 0.;
    for (int k = 0; k < p.npdf; ++k) {
        const PdfDesc &d = p.pdf[k];
        double t = 0.;
        if (d.kind == MCIG_PDF_GAUSS || d.kind == MCIG_PDF_EXP) {
            for (int i = 0; i < p.ndim; ++i) { t = t + proto_i_d(d.kind, x[i]); }
        } else {
            t = t + pdf_proto_scalar_d(p, d, x);
        }
        s = s - t;
    }
    return s;
}

template <class R>
__device__ void obs_eval(const KParams &p, const ObsDesc &o, const R *x, R *out, const float *blob = nullptr)
{
    const int nd = p.ndim;
    switch (o.kind) {
    case MCIG_OBS_LOGPDF: { // a dependent observable: reads the sampling functions
        if constexpr (std::is_same<R, double>::value) { out[0] = logpdf_d(p, x); }
        else {
            float s = 0.f;
            for (int k = 0; k < p.npdf; ++k) { s += pdf_logp_f(p, p.pdf[k], x, blob ? blob : p.fblob); }
            out[0] = s;
        }
        break;
    }
    case MCIG_OBS_X2SUM: { // X2Sum (:424-430)
        R s = (R)0;
        for (int i = 0; i < nd; ++i) { s = s + x[i] * x[i]; }
        out[0] = s;
        break;
    }
    case MCIG_OBS_XND: // XND (:344-347)
        for (int i = 0; i < nd; ++i) { out[i] = x[i]; }
        break;
    case MCIG_OBS_X2: // X2 (:445-450)
        for (int i = 0; i < nd; ++i) { out[i] = x[i] * x[i]; }
        break;
    case MCIG_OBS_X2MEAN: { // XSquared (:269-272)
        R s = x[0] * x[0];
        for (int i = 1; i < nd; ++i) { s = s + x[i] * x[i]; }
        out[0] = s / (R)nd;
        break;
    }
    case MCIG_OBS_CONST: out[0] = (R)p.params[o.poff]; break; // Constval (:385-388)
    case MCIG_OBS_XI: out[0] = x[(int)p.params[o.poff]]; break;
    case MCIG_OBS_POLYNOM: { // Polynom (:403-409)
        R s = (R)0;
        for (int i = 0; i < nd; ++i) { s = s + x[i]; }
        out[0] = s;
        break;
    }
    case MCIG_OBS_X2BLOCK: {
        const double *pp = p.params + o.poff;
        const int nb = (int)pp[0];
        for (int k = 0; k < nb; ++k) {
            R s = (R)0;
            for (int i = (int)pp[1 + k]; i < (int)pp[2 + k]; ++i) { s = s + x[i] * x[i]; }
            out[k] = s;
        }
        break;
    }
    case MCIG_OBS_GAUSSX2: { // GaussXSquared (:287-293); normf computed on the host
        R r2 = x[0] * x[0];
        for (int i = 1; i < nd; ++i) { r2 = r2 + x[i] * x[i]; }
        out[0] = exp(-r2) * r2 * (R)p.params[o.poff];
        break;
    }
    default: break;
    }
}

// ------------------------------------------------------------------------
// accumulator sums
// ------------------------------------------------------------------------
template <bool KAHAN> struct AccSlot;
template <> struct AccSlot<false> {
    double s;
    __device__ __forceinline__ void zero() { s = 0.; }
    __device__ __forceinline__ void add(double v) { s = s + v; }
    __device__ __forceinline__ double get() const { return s; }
};
template <> struct AccSlot<true> {
    float s, c;
    __device__ __forceinline__ void zero() { s = 0.f; c = 0.f; }
    __device__ __forceinline__ void add(float v)
    { // Kahan compensated summation
        const float y = v - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double get() const { return (double)s - (double)c; }
};

// ------------------------------------------------------------------------
// the sampler
// ------------------------------------------------------------------------
// proto values of plugin sampling functions: protoold / protonew of the main chain's (upo,
// upn) and of MultiStepMove's sub-pdfs (mpo, mpn), the k-th at k * max_nproto; an empty base
// of the built-in kernels
template <class R, int CAP, int PCAP, bool ON> struct UserProtoStore {
    R upo[CAP], upn[CAP], mpo[CAP], mpn[CAP];
    R uprep[PCAP]; // observationCallback output of each plugin pdf, the k-th at k * max_nprep
};
template <class R, int CAP, int PCAP> struct UserProtoStore<R, CAP, PCAP, false> {
    static constexpr R *upo = nullptr, *upn = nullptr, *mpo = nullptr, *mpn = nullptr, *uprep = nullptr;
};
// a user trial move's protoold / protonew and the changed indices it reports
template <class R, int CAP, bool ON> struct UserMoveStore {
    R vpo[CAP], vpn[CAP];
    int chidx[MCIG_MAXDIM];
};
template <class R, int CAP> struct UserMoveStore<R, CAP, false> {
    static constexpr R *vpo = nullptr, *vpn = nullptr;
    static constexpr int *chidx = nullptr;
};

// U: the plugin's functor lists (mcig_plugin.cuh); mcig::NoPlugin for the built-in kernels
template <class R, int RNG, bool KAHAN, class U = mcig::NoPlugin>
struct GenericSampler : UserProtoStore<R, MCIG_MAXPDF * U::max_nproto, MCIG_MAXPDF * U::max_nprep, (U::npdf > 0)>,
                        UserMoveStore<R, U::move_max_nproto, (U::nmove > 0)> {
    static constexpr bool EXACT = std::is_same<R, double>::value;
    static constexpr int NV = 2 * MCIG_MAXDIM + 8;
    using AccV = typename std::conditional<KAHAN, float, double>::type;
    static constexpr bool USER_PDF = U::npdf > 0;
    static constexpr bool USER_OBS = U::nobs > 0;
    static constexpr bool USER_MOVE = U::nmove > 0;
    static constexpr int MP = U::max_nproto; // proto values per plugin pdf

    const KParams &p;
    const int c;
    const float *blob;
    R x[MCIG_MAXDIM];
    R xn[MCIG_MAXDIM];
    R w[MCIG_MAXDIM];
    R st[MCIG_MAXTYPES];
    R lp[MCIG_MAXPDF]; // double: scalar proto per pdf at x; float: log density per pdf at x
    PhiloxCtx ph;
    uint64_t ctr;
    int64_t tpos, tlen;
    const double *tape;
    int tape_err;

    __device__ GenericSampler(const KParams &pp, int cc, const float *bl) : p(pp), c(cc), blob(bl), tape_err(0)
    {
        for (int i = 0; i < p.ndim; ++i) { x[i] = (R)p.x[(size_t)i * p.nchains + c]; }
        for (int t = 0; t < p.ntypes; ++t) { st[t] = (R)p.step[(size_t)t * p.nchains + c]; }
        ctr = 0;
        tpos = 0;
        tlen = 0;
        tape = nullptr;
        if constexpr (RNG == RNG_PHILOX) {
            ctr = p.ctr[c];
            ph.k0 = p.key0;
            ph.k1 = p.key1;
            ph.chain = (uint32_t)c;
        } else {
            tpos = p.tpos[c];
            tlen = p.tape_len[c];
            tape = p.tape + (size_t)c * p.tape_stride;
        }
    }

    __device__ __forceinline__ double tape_next()
    {
        if (tpos < tlen) { return tape[tpos++]; }
        tape_err = 1;
        return 0.5;
    }

    __device__ __forceinline__ void begin_step()
    {
        if constexpr (RNG == RNG_PHILOX) {
            ph.s0 = (uint32_t)ctr;
            ph.s1 = (uint32_t)(ctr >> 32);
        }
    }
    __device__ __forceinline__ void end_step()
    {
        if constexpr (RNG == RNG_PHILOX) { ++ctr; }
    }

    __device__ __forceinline__ R pdf_state(const PdfDesc &d, const R *pos)
    {
        if constexpr (EXACT) { return pdf_proto_scalar_d(p, d, pos); }
        else { return pdf_logp_f(p, d, pos, blob); }
    }

    __device__ __forceinline__ bool user_pdf(const PdfDesc &d) const
    {
        if constexpr (USER_PDF) { return d.kind >= MCIG_PDF_USER; }
        else { return false; }
    }
    __device__ __forceinline__ bool user_obs(const ObsDesc &o) const
    {
        if constexpr (USER_OBS) { return o.kind >= MCIG_OBS_USER; }
        else { return false; }
    }
    __device__ __forceinline__ mcig::UserArgs uargs(int poff, int np) const { return mcig::UserArgs{p.ndim, p.params + poff, np}; }

    // ProtoFunctionInterface::initializeProtoValues of a plugin sampling function (protonew = protoold)
    __device__ void user_init(const PdfDesc &d, const R *pos, R *po, R *pn)
    {
        U::proto(d.kind - MCIG_PDF_USER, uargs(d.poff, d.np), pos, po);
        for (int j = 0; j < d.nproto; ++j) { pn[j] = po[j]; }
    }
    // SamplingFunctionInterface::computeAcceptance of a plugin sampling function: updates pn
    // idx: the changed indices of a user trial move (nchanged of them), else NULL and [lo, hi)
    __device__ R user_accept(const PdfDesc &d, const R *xo, const R *xnew, bool partial, int lo, int hi, const R *po, R *pn,
                             const int *idx = nullptr, int nchanged = 0)
    {
        const mcig::UserWalker<R> w{xo, xnew, idx ? nchanged : hi - lo, lo, idx};
        return U::accept(d.kind - MCIG_PDF_USER, uargs(d.poff, d.np), w, partial, po, pn);
    }
    // newToOld (src, dst) = (pn, po) on acceptance, oldToNew = (po, pn) on rejection
    __device__ __forceinline__ static void copy_protos(const R *src, R *dst, int n)
    {
        for (int j = 0; j < n; ++j) { dst[j] = src[j]; }
    }
    // samplingFunction of a plugin pdf at its protos: the value (double) or its log (float)
    __device__ __forceinline__ R user_value(const PdfDesc &d, const R *pv)
    {
        const R v = U::sampling(d.kind - MCIG_PDF_USER, uargs(d.poff, d.np), pv);
        if constexpr (EXACT) { return v; }
        else { return logf(v); }
    }

    // ProtoFunctionInterface::initializeProtoValues (ProtoFunctionInterface.cpp:40-44)
    __device__ void init_protos()
    {
        for (int k = 0; k < p.npdf; ++k) {
            if (user_pdf(p.pdf[k])) { user_init(p.pdf[k], x, this->upo + k * MP, this->upn + k * MP); }
            else { lp[k] = pdf_state(p.pdf[k], x); }
        }
        if constexpr (USER_MOVE) { // _trialMove->initializeProtoValues(xold) (MCIntegrator.cpp:261)
            if (p.umove_nproto > 0) {
                U::move_proto(p.umove, uargs(p.umove_poff, p.umove_np), (const R *)x, this->vpo);
                copy_protos(this->vpo, this->vpn, p.umove_nproto);
            }
        }
    }

    // TrialMoveInterface::computeTrialMove of a plugin move: xn = the proposal (xn == x on
    // entry); returns the move's acceptance factor (double) or its log (float); nch and the
    // changed indices in chidx, lo/hi their hull
    template <bool ON = USER_MOVE> __device__ R user_move(int &nch, int &lo, int &hi)
    {
        for (int i = 0; i < p.ndim; ++i) { xn[i] = x[i]; }
        mcig::UserMoveWalker<R> mw{p.ndim, x, xn, p.ndim, this->chidx};
        mcig::UserRng<R> rng;
        rng.blk = 0;
        rng.iblk = 0;
        rng.nw = 0;
        rng.has_spare = false;
        rng.ncache = 0;
        rng.cache_srrd = -1;
        rng.spare = (R)0;
        rng.tape = nullptr;
        rng.tpos = &tpos;
        rng.tlen = tlen;
        rng.err = &tape_err;
        if constexpr (RNG == RNG_TAPE) { rng.tape = tape; }
        else { rng.ph = ph; }
        const R a = U::move(p.umove, uargs(p.umove_poff, p.umove_np), mw, st, rng, this->vpo, this->vpn);
        nch = mw.nchanged < 0 ? 0 : (mw.nchanged > p.ndim ? p.ndim : mw.nchanged);
        if (nch >= p.ndim) {
            lo = 0;
            hi = p.ndim;
        } else if (nch == 0) {
            lo = 0;
            hi = 0;
        } else {
            lo = this->chidx[0];
            hi = this->chidx[nch - 1] + 1;
        }
        if constexpr (EXACT) { return a; }
        else { return logf(a); }
    }

    // draw j of the move group (substep, TAG_MOVE): coordinate-indexed for Philox
    __device__ __forceinline__ void move_group(int substep, int srrd, int b, R *d)
    {
        move_draws_srrd<R>(ph.block(substep, TAG_MOVE, b), srrd, d);
    }

    // SRRDAllMove::trialMove (SRRDAllMove.hpp:67-80): xn = x + step(type(i)) * d_i
    __device__ void all_move(int srrd)
    {
        constexpr int CPB = Cpb<R>::v;
        R d[CPB];
        for (int i = 0; i < p.ndim; ++i) {
            R v;
            if constexpr (RNG == RNG_TAPE) { v = (R)tape_next(); }
            else {
                if (i % CPB == 0) { move_group(0, srrd, i / CPB, d); }
                v = d[i % CPB];
            }
            xn[i] = x[i];
            xn[i] = xn[i] + step_of_rt<R>(p, st, i) * v;
        }
    }

    // SRRDVecMove::trialMove (SRRDVecMove.hpp:75-96) from pos into xn; returns the first index
    // copy_all false: xn already equals pos outside the moved vector (MultiStepMove keeps it so)
    __device__ int vec_move(const R *pos, int substep, int srrd, int veclen, bool copy_all = true)
    {
        const int nvecs = p.ndim / veclen;
        int vidx;
        if constexpr (RNG == RNG_TAPE) {
            vidx = (int)tape_next();
            vidx = vidx < 0 ? 0 : (vidx >= nvecs ? nvecs - 1 : vidx);
        } else {
            // multiply-shift index; bias below nvecs / 2^32
            vidx = (int)__umulhi(ph.block(substep, TAG_INDEX, 0).a, (uint32_t)nvecs);
        }
        const int lo = vidx * veclen;
        const R s = step_of_rt<R>(p, st, lo);
        if (copy_all) {
            for (int i = 0; i < p.ndim; ++i) { xn[i] = pos[i]; }
        } else {
            for (int i = lo; i < lo + veclen; ++i) { xn[i] = pos[i]; }
        }
        constexpr int CPB = Cpb<R>::v;
        R d[CPB];
        for (int i = lo; i < lo + veclen; ++i) {
            R v;
            if constexpr (RNG == RNG_TAPE) { v = (R)tape_next(); }
            else {
                if (i == lo || i % CPB == 0) { move_group(substep, srrd, i / CPB, d); }
                v = d[i % CPB];
            }
            xn[i] = xn[i] + s * v;
        }
        return lo;
    }

    __device__ __forceinline__ R accept_u(int substep)
    {
        if constexpr (RNG == RNG_TAPE) { return (R)tape_next(); }
        else { return accept_draw<R>(ph.block(substep, TAG_ACCEPT, 0)); }
    }

    // MultiStepMove::trialMove (src/MultiStepMove.cpp:6-47): nested chain on the
    // sub-pdfs; returns oldPDF/newPDF (double) or its log (float); xn = end point.
    __device__ R multistep()
    {
        // w: the sub-chain's walker; xn equals w outside the vector a sub-step moves, so a
        // sub-step touches only veclen coordinates
        for (int i = 0; i < p.ndim; ++i) { w[i] = x[i]; xn[i] = x[i]; }
        R sp[MCIG_MAXPDF];
        for (int k = 0; k < p.ms_npdf; ++k) {
            if (user_pdf(p.ms_pdf[k])) {
                user_init(p.ms_pdf[k], w, this->mpo + k * MP, this->mpn + k * MP);
                sp[k] = user_value(p.ms_pdf[k], this->mpo + k * MP);
            } else {
                sp[k] = pdf_state(p.ms_pdf[k], w);
            }
        }
        R oldv;
        if constexpr (EXACT) {
            oldv = 1.;
            for (int k = 0; k < p.ms_npdf; ++k) {
                oldv *= user_pdf(p.ms_pdf[k]) ? sp[k] : pdf_value_d(p, p.ms_pdf[k], w, sp[k]);
            }
        } else {
            oldv = 0.f;
            for (int k = 0; k < p.ms_npdf; ++k) { oldv += sp[k]; }
        }
        for (int s = 0; s < p.ms_nsteps; ++s) {
            const int lo = vec_move(w, 1 + s, p.ms_srrd, p.ms_veclen, false);
            const int hi = lo + p.ms_veclen;
            R spn[MCIG_MAXPDF];
            bool acc;
            if constexpr (EXACT) {
                double a = 1.;
                const bool partial = p.ms_veclen < p.ndim;
                for (int k = 0; k < p.ms_npdf; ++k) {
                    if (user_pdf(p.ms_pdf[k])) {
                        a *= user_accept(p.ms_pdf[k], w, xn, partial, lo, hi, this->mpo + k * MP, this->mpn + k * MP);
                        spn[k] = sp[k];
                        continue;
                    }
                    double pn = 0.;
                    a *= pdf_accept_d(p, p.ms_pdf[k], w, xn, partial, lo, hi, sp[k], pn);
                    spn[k] = pn;
                }
                acc = (accept_u(1 + s) <= a * 1.);
            } else {
                float dl = 0.f;
                const bool partial = p.ms_veclen < p.ndim;
                for (int k = 0; k < p.ms_npdf; ++k) {
                    float delta;
                    if (user_pdf(p.ms_pdf[k])) {
                        delta = logf(user_accept(p.ms_pdf[k], w, xn, partial, lo, hi, this->mpo + k * MP, this->mpn + k * MP));
                    } else if (!pdf_delta_f(p.ms_pdf[k], w, xn, lo, hi, delta)) {
                        delta = pdf_logp_f(p, p.ms_pdf[k], xn, blob) - sp[k];
                    }
                    spn[k] = sp[k] + delta;
                    dl += delta;
                }
                acc = (__log2f(accept_u(1 + s)) <= dl * 1.44269504f);
            }
            if (acc) {
                for (int i = lo; i < hi; ++i) { w[i] = xn[i]; }
                for (int k = 0; k < p.ms_npdf; ++k) { sp[k] = spn[k]; }
            } else {
                for (int i = lo; i < hi; ++i) { xn[i] = w[i]; }
            }
            if constexpr (USER_PDF) {
                for (int k = 0; k < p.ms_npdf; ++k) {
                    if (!user_pdf(p.ms_pdf[k])) { continue; }
                    if (acc) { copy_protos(this->mpn + k * MP, this->mpo + k * MP, p.ms_pdf[k].nproto); }
                    else { copy_protos(this->mpo + k * MP, this->mpn + k * MP, p.ms_pdf[k].nproto); }
                }
            }
        }
        // xn == w: the end point of the sub-chain
        if constexpr (EXACT) {
            double newv = 1.;
            for (int k = 0; k < p.ms_npdf; ++k) {
                newv *= user_pdf(p.ms_pdf[k]) ? user_value(p.ms_pdf[k], this->mpo + k * MP)
                                              : pdf_value_d(p, p.ms_pdf[k], w, sp[k]);
            }
            return oldv / newv;
        } else {
            float newv = 0.f;
            for (int k = 0; k < p.ms_npdf; ++k) {
                newv += user_pdf(p.ms_pdf[k]) ? user_value(p.ms_pdf[k], this->mpo + k * MP) : sp[k];
            }
            return oldv - newv;
        }
    }

    // MCI::doStepMRT2 (MCIntegrator.cpp:326-360)
    __device__ bool step_mrt2(int movetype)
    {
        begin_step();
        R moveAcc = EXACT ? (R)1 : (R)0;
        bool partial = false;
        int lo = 0, hi = p.ndim;
        const int *uidx = nullptr; // the changed indices of a user move with nchanged < ndim
        int nch = 0;
        if (movetype == MCIG_MOVE_ALL) {
            all_move(p.srrd);
        } else if (movetype == MCIG_MOVE_VEC) {
            lo = vec_move(x, 0, p.srrd, p.veclen);
            hi = lo + p.veclen;
            partial = p.veclen < p.ndim;
        } else if (movetype == MCIG_MOVE_USER) {
            if constexpr (USER_MOVE) {
                moveAcc = user_move(nch, lo, hi);
                partial = nch < p.ndim;
                if (partial) { uidx = this->chidx; }
            }
        } else {
            moveAcc = multistep();
        }
        if (p.periodic) { // applyDomain on the changed indices (xn == x elsewhere in [lo, hi))
            if (uidx) {
                for (int j = 0; j < nch; ++j) { periodic_wrap(xn[uidx[j]], p.lb[uidx[j]], p.ub[uidx[j]]); }
            } else {
                for (int i = lo; i < hi; ++i) { periodic_wrap(xn[i], p.lb[i], p.ub[i]); }
            }
        }
        R lpn[MCIG_MAXPDF];
        bool acc;
        if constexpr (EXACT) {
            double a = 1.;
            for (int k = 0; k < p.npdf; ++k) {
                double pn = lp[k];
                if (user_pdf(p.pdf[k])) {
                    a *= user_accept(p.pdf[k], x, xn, partial, lo, hi, this->upo + k * MP, this->upn + k * MP, uidx, nch);
                } else {
                    a *= pdf_accept_d(p, p.pdf[k], x, xn, partial, lo, hi, lp[k], pn);
                }
                lpn[k] = pn;
            }
            acc = (accept_u(0) <= a * moveAcc);
        } else {
            float dl = moveAcc;
            for (int k = 0; k < p.npdf; ++k) {
                if (user_pdf(p.pdf[k])) {
                    lpn[k] = lp[k];
                    dl += logf(user_accept(p.pdf[k], x, xn, partial, lo, hi, this->upo + k * MP, this->upn + k * MP, uidx, nch));
                    continue;
                }
                lpn[k] = pdf_logp_f(p, p.pdf[k], xn, blob);
                dl += lpn[k] - lp[k];
            }
            acc = (__log2f(accept_u(0)) <= dl * 1.44269504f);
        }
        if (acc) {
            for (int i = lo; i < hi; ++i) { x[i] = xn[i]; }
            for (int k = 0; k < p.npdf; ++k) { lp[k] = lpn[k]; }
        }
        if constexpr (USER_PDF) { // newToOld / oldToNew (ProtoFunctionInterface.cpp:46-56)
            for (int k = 0; k < p.npdf; ++k) {
                if (!user_pdf(p.pdf[k])) { continue; }
                if (acc) { copy_protos(this->upn + k * MP, this->upo + k * MP, p.pdf[k].nproto); }
                else { copy_protos(this->upo + k * MP, this->upn + k * MP, p.pdf[k].nproto); }
            }
        }
        if constexpr (USER_MOVE) { // _trialMove->newToOld() / oldToNew()
            if (movetype == MCIG_MOVE_USER && p.umove_nproto > 0) {
                if (acc) { copy_protos(this->vpn, this->vpo, p.umove_nproto); }
                else { copy_protos(this->vpo, this->vpn, p.umove_nproto); }
            }
        }
        end_step();
        return acc;
    }

    // MCI::doStepRandom (MCIntegrator.cpp:362-376) in the periodic box
    __device__ bool step_random()
    {
        begin_step();
        constexpr int CPB = Cpb<R>::v;
        R d[CPB];
        for (int i = 0; i < p.ndim; ++i) {
            R u;
            if constexpr (RNG == RNG_TAPE) { u = (R)tape_next(); }
            else {
                if (i % CPB == 0) { move_group(0, MCIG_SRRD_UNIFORM, i / CPB, d); }
                u = (d[i % CPB] + (R)1) * (R)0.5;
            }
            xn[i] = u;
        }
        for (int i = 0; i < p.ndim; ++i) { x[i] = (R)p.lb[i] + xn[i] * (R)(p.ub[i] - p.lb[i]); }
        end_step();
        return true;
    }

    __device__ __forceinline__ bool step(int movetype) { return p.npdf > 0 ? step_mrt2(movetype) : step_random(); }

    __device__ void store_state()
    {
        for (int i = 0; i < p.ndim; ++i) { p.x[(size_t)i * p.nchains + c] = (double)x[i]; }
        for (int t = 0; t < p.ntypes; ++t) { p.step[(size_t)t * p.nchains + c] = (double)st[t]; }
        if constexpr (RNG == RNG_PHILOX) { p.ctr[c] = ctr; }
        else { p.tpos[c] = tpos; }
        if (tape_err) { atomicOr(p.status, 1); }
    }

    // MCI::sample(npoints) (MCIntegrator.cpp:273-288)
    __device__ void run_steps(int movetype, int64_t n)
    {
        init_protos();
        int64_t na = 0;
        for (int64_t r = 0; r < n; ++r) { na += step(movetype) ? 1 : 0; }
        p.nacc[c] = na;
        p.nrej[c] = n - na;
    }

    // the dependencies a dependent plugin observable reads at the walker x: the plugin pdfs'
    // proto values and observationCallback data (SamplingFunctionContainer::prepareObservation,
    // SamplingFunctionContainer.cpp:50-55), and the step's observable values so far
    __device__ void prepare_deps(mcig::UserDeps<R> &d, const R *vals)
    {
        d.npdf = p.npdf;
        d.obsvals = vals;
        for (int k = 0; k < MCIG_MAXPDF; ++k) {
            d.nproto[k] = 0;
            d.proto[k] = nullptr;
            d.prep[k] = nullptr;
        }
        if constexpr (USER_PDF) {
            for (int k = 0; k < p.npdf; ++k) {
                if (!user_pdf(p.pdf[k])) { continue; }
                d.nproto[k] = p.pdf[k].nproto;
                d.proto[k] = this->upo + k * MP;
                R *pr = this->uprep + k * U::max_nprep;
                if (U::prepare(p.pdf[k].kind - MCIG_PDF_USER, uargs(p.pdf[k].poff, p.pdf[k].np), (const R *)x, d.proto[k], pr)) {
                    d.prep[k] = pr;
                }
            }
        }
    }

    // MCI::sample(npoints, container, flagMC) (MCIntegrator.cpp:290-321) with the
    // accumulators: observable o is evaluated at the walker position after steps
    // r = 0, nskip, 2 nskip, ... (AccumulatorInterface.cpp:21-29, :99-114).  The
    // reference reuses the last values on rejected steps; a pure function of the
    // unchanged position gives the same values, so they are recomputed.
    __device__ void run_sample(int movetype, int64_t n)
    {
        init_protos();
        AccSlot<KAHAN> sums[NV];
        R vals[NV];
        for (int j = 0; j < p.nobsdim; ++j) { sums[j].zero(); }
        int64_t na = 0;
        int64_t dpos = 0; // next entry of the dump list (chain 0)
        // per observable: steps until its next accumulation (nskip), accumulation index,
        // accumulations left in the current block, block index - counters instead of
        // 64-bit divisions on every step
        int skipleft[MCIG_MAXOBS], bleft[MCIG_MAXOBS];
        int64_t kacc[MCIG_MAXOBS], bidx[MCIG_MAXOBS];
        for (int o = 0; o < p.nobs; ++o) {
            skipleft[o] = 0;
            bleft[o] = p.obs[o].bs;
            kacc[o] = 0;
            bidx[o] = 0;
        }
        mcig::UserDeps<R> deps;
        bool prepared = false;
        for (int64_t r = 0; r < n; ++r) {
            const bool a = step(movetype);
            prepared = false;
            if (c == 0 && dpos < p.ndump && r == p.dump_steps[dpos]) {
                for (int i = 0; i < p.ndim; ++i) { p.dump_x[dpos * p.ndim + i] = (double)x[i]; }
                ++dpos;
            }
            na += a ? 1 : 0;
            if (p.bits) { p.bits[(size_t)r * p.nchains + c] = a ? 1 : 0; }
            for (int o = 0; o < p.nobs; ++o) {
                const ObsDesc &od = p.obs[o];
                if (skipleft[o] > 0) { --skipleft[o]; continue; } // accumulate when nskip divides r
                skipleft[o] = od.nskip - 1;
                const int64_t k = kacc[o]++; // accumulation index r / nskip
                // plugin kernels keep every value of the step at its offset, for dependent observables
                R *const v = USER_OBS ? vals + od.voff : vals;
                if (user_obs(od)) {
                    if constexpr (U::any_deps) {
                        if (!prepared) { // SamplingFunctionContainer::prepareObservation at this walker
                            prepare_deps(deps, vals);
                            prepared = true;
                        }
                        U::observe_deps(od.kind - MCIG_OBS_USER, uargs(od.poff, od.np), (const R *)x, v, deps);
                    } else {
                        U::observe(od.kind - MCIG_OBS_USER, uargs(od.poff, od.np), (const R *)x, v);
                    }
                } else {
                    obs_eval<R>(p, od, x, v, blob);
                }
                if (od.acc == MCIG_ACC_FULL) { // FullAccumulator::_accumulate (FullAccumulator.cpp:14-18)
                    const size_t row = (size_t)(p.acc_offset + k);
                    if (od.full32) {
                        float *dst = (float *)od.data + row * od.nv * p.nchains + c;
                        for (int j = 0; j < od.nv; ++j) { dst[(size_t)j * p.nchains] = (float)v[j]; }
                    } else {
                        double *dst = (double *)od.data + row * od.nv * p.nchains + c;
                        for (int j = 0; j < od.nv; ++j) { dst[(size_t)j * p.nchains] = (double)v[j]; }
                    }
                } else {
                    for (int j = 0; j < od.nv; ++j) { sums[od.voff + j].add((AccV)v[j]); }
                    if (od.acc == MCIG_ACC_BLOCK && --bleft[o] == 0) { // blocksize divides k + 1
                        // block sum times 1./blocksize (BlockAccumulator.cpp:20-41)
                        bleft[o] = od.bs;
                        double *dst = (double *)od.data + (size_t)(bidx[o]++) * od.nv * p.nchains + c;
                        for (int j = 0; j < od.nv; ++j) {
                            dst[(size_t)j * p.nchains] = sums[od.voff + j].get() * od.inv_bs;
                            sums[od.voff + j].zero();
                        }
                    }
                }
            }
        }
        for (int o = 0; o < p.nobs; ++o) { // SimpleAccumulator::_finalize (SimpleAccumulator.cpp:22-29)
            const ObsDesc &od = p.obs[o];
            if (od.acc != MCIG_ACC_SIMPLE) { continue; }
            const double normf = 1. / (double)(1 + (n - 1) / od.nskip);
            double *dst = (double *)od.data + c;
            for (int j = 0; j < od.nv; ++j) { dst[(size_t)j * p.nchains] = sums[od.voff + j].get() * normf; }
        }
        p.nacc[c] = na;
        p.nrej[c] = n - na;
    }

    // MCI::findMRT2Step (MCIntegrator.cpp:87-168) for this chain alone
    __device__ void run_calibration(int movetype, int64_t MIN_STAT)
    {
        const int MIN_CONS = 5;
        const double TOLERANCE = 0.05;
        const double SMALLEST = 1.1754943508222875e-38; // numeric_limits<float>::min()
        int cons = 0, counter = 0;
        int64_t na = 0;
        while ((p.nfind < 0 && cons < MIN_CONS) || counter < p.nfind) {
            init_protos();
            na = 0;
            for (int64_t r = 0; r < MIN_STAT; ++r) { na += step(movetype) ? 1 : 0; }
            const double rate = (na > 0) ? (double)na / ((double)na + (double)(MIN_STAT - na)) : 0.;
            if (fabs(rate - p.target) < TOLERANCE) { ++cons; } else { cons = 0; }
            double f = rate / p.target;
            f = (f > 0.5) ? f : 0.5;
            f = (f < 2.) ? f : 2.;
            double sd[MCIG_MAXTYPES];
            for (int t = 0; t < p.ntypes; ++t) { sd[t] = (double)st[t] * f; } // scaleStepSizes
            if (movetype == MCIG_MOVE_USER) { // the move's getStepSizeIndex, folded into a limit per step size
                for (int t = 0; t < p.ntypes; ++t) {
                    const double lim = p.params[p.step_lim_off + t];
                    if (sd[t] > lim) { sd[t] = lim; }
                }
            } else {
                for (int i = 0; i < p.ndim; ++i) {
                    int t = 0;
                    while (t + 1 < p.ntypes && i >= p.typeEnds[t]) { ++t; }
                    const double lim = p.step_max_i ? p.step_max_i[i] : p.step_max;
                    if (sd[t] > lim) { sd[t] = lim; }
                }
            }
            for (int t = 0; t < p.ntypes; ++t) {
                if (sd[t] < SMALLEST) { sd[t] = SMALLEST; }
                st[t] = (R)sd[t];
            }
            ++counter;
            if (p.nfind < 0 && counter >= abs(p.nfind)) { break; }
        }
        p.nacc[c] = na;
        p.nrej[c] = (counter > 0) ? MIN_STAT - na : 0;
    }
};

template <class R, int RNG, bool KAHAN, class U = mcig::NoPlugin>
__global__ void __launch_bounds__(128) mcig_generic_kernel(const KParams p, int movetype)
{
    extern __shared__ float smem_blob[];
    for (int i = threadIdx.x; i < p.fblob_len; i += blockDim.x) { smem_blob[i] = p.fblob[i]; }
    __syncthreads();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= p.nchains) { return; }
    if (p.active && !p.active[c]) { return; }
    GenericSampler<R, RNG, KAHAN, U> s(p, c, smem_blob);
    if (p.mode == KMODE_CALIB) { s.run_calibration(movetype, p.nsteps); }
    else if (p.mode == KMODE_SAMPLE) { s.run_sample(movetype, p.nsteps); }
    else { s.run_steps(movetype, p.nsteps); }
    s.store_state();
}
