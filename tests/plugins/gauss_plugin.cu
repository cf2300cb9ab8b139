// Test plugin: user functors written the way a user of the reference writes
// SamplingFunctionInterface / ObservableFunctionInterface / TrialMoveInterface classes, with
// the arithmetic of the reference's test classes (test/common/TestMCIFunctions.hpp) and
// built-in moves, so that integrals with them equal integrals with the built-in kinds bit
// for bit.
#include <mcig/plugin.cuh>

// exp(-sum_i x_i^2) with one proto value per index (Gauss, TestMCIFunctions.hpp:151-190)
struct IndexGauss {
    static constexpr int max_nproto = 64;
    static int nproto(int ndim) { return ndim; }
    template <class R> __device__ static void protoFunction(const mcig::UserArgs &a, const R *in, R *pv)
    {
        for (int i = 0; i < a.ndim; ++i) { pv[i] = in[i] * in[i]; }
    }
    template <class R> __device__ static R samplingFunction(const mcig::UserArgs &a, const R *pv)
    {
        R s = (R)0;
        for (int i = 0; i < a.ndim; ++i) { s = s + pv[i]; }
        return exp(-s);
    }
    template <class R> __device__ static R acceptanceFunction(const mcig::UserArgs &a, const R *po, const R *pn)
    {
        R e = (R)0;
        for (int i = 0; i < a.ndim; ++i) { e = e + po[i]; }
        R f = (R)0;
        for (int i = 0; i < a.ndim; ++i) { f = f + pn[i]; }
        e = e - f;
        return exp(e);
    }
    template <class R>
    __device__ static R updatedAcceptance(const mcig::UserArgs &, const mcig::UserWalker<R> &w, const R *po, R *pn)
    {
        R e = (R)0;
        for (int j = 0; j < w.nchanged; ++j) {
            const int i = w.changed(j);
            pn[i] = w.xnew[i] * w.xnew[i];
            e = e + (pn[i] - po[i]);
        }
        return exp(-e);
    }
    // SamplingFunctionInterface::observationCallback (:104): what it prepares for the dependent
    // observables at an observed walker, here the gradient of log p, -2 x_i
    static constexpr int max_nprep = 64;
    template <class R> __device__ static void observationCallback(const mcig::UserArgs &a, const R *in, const R *, R *prep)
    {
        for (int i = 0; i < a.ndim; ++i) { prep[i] = (R)(-2) * in[i]; }
    }
};

// exp(-sum_i x_i^2) with a single proto value (ThreeDimGaussianPDF, :123-148, any ndim);
// no updatedAcceptance: partial moves recompute the proto value
struct SumGauss {
    static constexpr int max_nproto = 1;
    static int nproto(int) { return 1; }
    template <class R> __device__ static void protoFunction(const mcig::UserArgs &a, const R *in, R *pv)
    {
        R s = in[0] * in[0];
        for (int i = 1; i < a.ndim; ++i) { s = s + in[i] * in[i]; }
        pv[0] = s;
    }
    template <class R> __device__ static R samplingFunction(const mcig::UserArgs &, const R *pv) { return exp(-pv[0]); }
    template <class R> __device__ static R acceptanceFunction(const mcig::UserArgs &, const R *po, const R *pn)
    {
        return exp(-pn[0] + po[0]);
    }
};

// exp(-c sum_{b0<=i<b1} x_i^2), parameters [b0, b1, c]
struct ScaledBlockGauss {
    static constexpr int max_nproto = 1;
    static int nproto(int) { return 1; }
    template <class R> __device__ static void protoFunction(const mcig::UserArgs &a, const R *in, R *pv)
    {
        R s = (R)0;
        for (int i = (int)a.params[0]; i < (int)a.params[1]; ++i) { s = s + in[i] * in[i]; }
        pv[0] = s * (R)a.params[2];
    }
    template <class R> __device__ static R samplingFunction(const mcig::UserArgs &, const R *pv) { return exp(-pv[0]); }
    template <class R> __device__ static R acceptanceFunction(const mcig::UserArgs &, const R *po, const R *pn)
    {
        return exp(-pn[0] + po[0]);
    }
};

// sum_i x_i^2 (X2Sum, :415-433)
struct SquaredNorm {
    static int nobs(int) { return 1; }
    template <class R> __device__ static void observableFunction(const mcig::UserArgs &a, const R *in, R *out)
    {
        R s = (R)0;
        for (int i = 0; i < a.ndim; ++i) { s = s + in[i] * in[i]; }
        out[0] = s;
    }
};

// x_i (XND, :335-350)
struct Position {
    static int nobs(int ndim) { return ndim; }
    template <class R> __device__ static void observableFunction(const mcig::UserArgs &a, const R *in, R *out)
    {
        for (int i = 0; i < a.ndim; ++i) { out[i] = in[i]; }
    }
};

// x_i + params[0]: an observable with a parameter
struct ShiftedPosition {
    static int nobs(int ndim) { return ndim; }
    template <class R> __device__ static void observableFunction(const mcig::UserArgs &a, const R *in, R *out)
    {
        for (int i = 0; i < a.ndim; ++i) { out[i] = in[i] + (R)a.params[0]; }
    }
};

// Dependent observables (DependentObservableInterface.hpp:24-53):
// log of the product of the plugin sampling functions from their proto values at the walker,
// -sum_k sum_i protov_k[i] (the index-proto Gauss's log density; the built-in LOGPDF order)
struct LogPdfFromProtos {
    static int nobs(int) { return 1; }
    template <class R>
    __device__ static void observableFunction(const mcig::UserArgs &, const R *, R *out, const mcig::UserDeps<R> &d)
    {
        R s = (R)0;
        for (int k = 0; k < d.npdf; ++k) {
            if (!d.proto[k]) { continue; }
            R t = (R)0;
            for (int i = 0; i < d.nproto[k]; ++i) { t = t + d.proto[k][i]; }
            s = s - t;
        }
        out[0] = s;
    }
};

// the first sampling function's prepared data (its observationCallback: the gradient of log p)
struct PreparedGradient {
    static int nobs(int ndim) { return ndim; }
    template <class R>
    __device__ static void observableFunction(const mcig::UserArgs &a, const R *, R *out, const mcig::UserDeps<R> &d)
    {
        for (int i = 0; i < a.ndim; ++i) { out[i] = d.prep[0] ? d.prep[0][i] : (R)0; }
    }
};

// the square of the step's first observable value (an earlier observable, nskip synced)
struct SquareOfFirst {
    static int nobs(int) { return 1; }
    template <class R>
    __device__ static void observableFunction(const mcig::UserArgs &, const R *, R *out, const mcig::UserDeps<R> &d)
    {
        out[0] = d.obsvals[0] * d.obsvals[0];
    }
};

// Trial moves (TrialMoveInterface, include/mci/TrialMoveInterface.hpp:18-75)

// x' = x + s z, z ~ N(0, I): the arithmetic and draws of SRRDAllMove with the normal
// distribution (SRRDAllMove.hpp:67-80), one step size
struct GaussAllMove {
    static int nstep(const mcig::UserArgs &) { return 1; }
    static double step0(const mcig::UserArgs &, int) { return 0.05; }
    static int step_index(const mcig::UserArgs &, int) { return 0; }
    static double change_rate(const mcig::UserArgs &) { return 1.; }
    template <class R>
    __device__ static R trialMove(const mcig::UserArgs &a, mcig::UserMoveWalker<R> &w, const R *steps,
                                  mcig::UserRng<R> &rng, const R *, R *)
    {
        for (int i = 0; i < a.ndim; ++i) { w.xnew[i] = w.xold[i] + steps[0] * rng.normal(); }
        w.nchanged = a.ndim;
        return (R)1;
    }
};

// one coordinate, uniform on [-s, s): SRRDVecMove with vector length 1 and the uniform
// distribution (SRRDVecMove.hpp:75-96): index first, then the displacement
struct SingleIndexMove {
    static int nstep(const mcig::UserArgs &) { return 1; }
    static double step0(const mcig::UserArgs &, int) { return 0.05; }
    static int step_index(const mcig::UserArgs &, int) { return 0; }
    static double change_rate(const mcig::UserArgs &a) { return 1. / a.ndim; }
    template <class R>
    __device__ static R trialMove(const mcig::UserArgs &a, mcig::UserMoveWalker<R> &w, const R *steps,
                                  mcig::UserRng<R> &rng, const R *, R *)
    {
        const int i = rng.index(a.ndim);
        w.xnew[i] = w.xold[i] + steps[0] * rng.draw(MCIG_SRRD_UNIFORM);
        w.nchanged = 1;
        w.changedIdx[0] = i;
        return (R)1;
    }
};

// two coordinates half the dimension apart (i and i + ndim/2 mod ndim, not adjacent), each
// with a Gaussian displacement; the first half of the coordinates has step size 0, the
// second half step size 1 (ndim >= 2)
struct PairMove {
    static int nstep(const mcig::UserArgs &) { return 2; }
    static double step0(const mcig::UserArgs &, int t) { return t == 0 ? 0.05 : 0.1; }
    static int step_index(const mcig::UserArgs &a, int xidx) { return xidx < a.ndim / 2 ? 0 : 1; }
    static double change_rate(const mcig::UserArgs &a) { return 2. / a.ndim; }
    template <class R>
    __device__ static R trialMove(const mcig::UserArgs &a, mcig::UserMoveWalker<R> &w, const R *steps,
                                  mcig::UserRng<R> &rng, const R *, R *)
    {
        const int h = a.ndim / 2;
        const int i = rng.index(a.ndim);
        const int j = (i + h) % a.ndim;
        const int lo = i < j ? i : j, hi = i < j ? j : i;
        w.xnew[lo] = w.xold[lo] + steps[lo < h ? 0 : 1] * rng.normal();
        w.xnew[hi] = w.xold[hi] + steps[hi < h ? 0 : 1] * rng.normal();
        w.nchanged = 2;
        w.changedIdx[0] = lo;
        w.changedIdx[1] = hi;
        return (R)1;
    }
};

// independence proposal x' ~ N(0, sigma^2 I), sigma = params[0]: not symmetric, so the move's
// acceptance factor is q(x) / q(x') = exp(|x'|^2 / (2 sigma^2) - |x|^2 / (2 sigma^2)), with
// the proto value |x|^2 / (2 sigma^2) kept for the old and the new position; no step sizes
struct IndependenceMove {
    static constexpr int max_nproto = 1;
    static int nproto(int) { return 1; }
    static int nstep(const mcig::UserArgs &) { return 0; }
    static double step0(const mcig::UserArgs &, int) { return 0.; }
    static int step_index(const mcig::UserArgs &, int) { return 0; }
    static double change_rate(const mcig::UserArgs &) { return 1.; }
    template <class R> __device__ static void protoFunction(const mcig::UserArgs &a, const R *x, R *pv)
    {
        R s = (R)0;
        for (int i = 0; i < a.ndim; ++i) { s = s + x[i] * x[i]; }
        pv[0] = s / (R)(2. * a.params[0] * a.params[0]);
    }
    template <class R>
    __device__ static R trialMove(const mcig::UserArgs &a, mcig::UserMoveWalker<R> &w, const R *,
                                  mcig::UserRng<R> &rng, const R *po, R *pn)
    {
        const R sg = (R)a.params[0];
        for (int i = 0; i < a.ndim; ++i) { w.xnew[i] = sg * rng.normal(); }
        w.nchanged = a.ndim;
        protoFunction(a, (const R *)w.xnew, pn);
        return exp(pn[0] - po[0]);
    }
};

using TestPdfs = mcig::PdfList<IndexGauss, SumGauss, ScaledBlockGauss>;
using TestObss = mcig::ObsList<SquaredNorm, Position, ShiftedPosition, LogPdfFromProtos, PreparedGradient, SquareOfFirst>;
using TestMoves = mcig::MoveList<GaussAllMove, SingleIndexMove, PairMove, IndependenceMove>;
MCIG_PLUGIN_MOVES(TestPdfs, TestObss, TestMoves)
