// mcig_plugin.cuh -- user sampling functions and observables as device types.
//
// The reference takes user code as C++ classes derived from SamplingFunctionInterface
// (include/mci/SamplingFunctionInterface.hpp:37-104: protoFunction, samplingFunction,
// acceptanceFunction, optional updatedAcceptance) and ObservableFunctionInterface
// (include/mci/ObservableFunctionInterface.hpp:24-60: observableFunction).  On the device
// the same four functions are static members of a struct, templated on the walker type R
// (double: the reference's arithmetic; float: the float path), and a plugin is a shared
// library that instantiates the general sampling kernel over a list of such structs
// (include/mcig/plugin.cuh).  A functor of the plugin is addressed by kind
// MCIG_PDF_USER + k / MCIG_OBS_USER + k, k its position in the list.
//
// Sampling function struct:
//   static constexpr int max_nproto;                     // compile-time bound of nproto
//   static int nproto(int ndim);                          // proto values (host and device)
//   template <class R> __device__ static void protoFunction(const UserArgs &, const R *x, R *protov);
//   template <class R> __device__ static R samplingFunction(const UserArgs &, const R *protov);
//   template <class R> __device__ static R acceptanceFunction(const UserArgs &, const R *protoold, const R *protonew);
//   optional:
//   template <class R> __device__ static R updatedAcceptance(const UserArgs &, const UserWalker<R> &,
//                                                             const R *protoold, R *protonew);
//   static constexpr int max_nprep;                     // with observationCallback: its values
//   template <class R> __device__ static void observationCallback(const UserArgs &, const R *x,
//                                                                  const R *protov, R *prep);
// Trial move struct (TrialMoveInterface, include/mci/TrialMoveInterface.hpp:18-75), host part
// on the handle's parameters (UserArgs::params, host memory there):
//   static int nstep(const UserArgs &);                  // getNStepSizes (0 .. MCIG_MAXTYPES)
//   static double step0(const UserArgs &, int t);         // initial step size t
//   static int step_index(const UserArgs &, int xidx);    // getStepSizeIndex
//   static double change_rate(const UserArgs &);          // getChangeRate
//   device part:
//   template <class R> __device__ static R trialMove(const UserArgs &, UserMoveWalker<R> &w,
//                                                     const R *steps, UserRng<R> &rng,
//                                                     const R *protoold, R *protonew);
//   optional, for a move with proto values (ProtoFunctionInterface):
//   static constexpr int max_nproto; static int nproto(int ndim);
//   template <class R> __device__ static void protoFunction(const UserArgs &, const R *x, R *protov);
// Observable struct:
//   static int nobs(int ndim);
//   template <class R> __device__ static void observableFunction(const UserArgs &, const R *x, R *out);
//   or, for an observable that depends on the sampling functions or earlier observables:
//   template <class R> __device__ static void observableFunction(const UserArgs &, const R *x, R *out,
//                                                                 const UserDeps<R> &deps);
#pragma once

#include <type_traits>
#include <utility>

#include "mcig_common.cuh"

namespace mcig {

// a functor's view of its configuration: the parameters given with
// addSamplingFunction / addObservable, as doubles
struct UserArgs {
    int ndim;
    const double *params;
    int nparams;
};

// WalkerState (include/mci/WalkerState.hpp) of a partial move: xold/xnew and the changed
// coordinates changed(0) < changed(1) < ... < changed(nchanged - 1) (the reference's
// changedIdx): lo, lo + 1, ... for the built-in moves (idx NULL), the list a user trial
// move reported otherwise
template <class R> struct UserWalker {
    const R *xold;
    const R *xnew;
    int nchanged;
    int lo;
    const int *idx;
    __device__ __forceinline__ int changed(int j) const { return idx ? idx[j] : lo + j; }
};

// WalkerState as a user trial move sees it (TrialMoveInterface::trialMove): xnew equals xold
// on entry; the move writes xnew, nchanged and, when nchanged < ndim, the ascending changed
// indices changedIdx[0 .. nchanged)
template <class R> struct UserMoveWalker {
    int ndim;
    const R *xold;
    R *xnew;
    int nchanged;
    int *changedIdx;
};

// The random numbers of a user trial move (the reference hands the move MCI's mt19937_64,
// TrialMoveInterface::getRGen).  Philox: the step's blocks (substep 0, TAG_MOVE, b = 0, 1, ...)
// in order, 4 words each, and for index() the blocks (0, TAG_INDEX, b); a recorded tape (FP64
// replay): every call returns the next recorded value, which is the value the reference's
// distribution call returned in the recorded run.
//   bits()      32 random bits
//   uniform()   [0, 1): 24 bits (float), 53 bits (double)
//   normal()    N(0, 1), Box-Muller pairs (the second value of a pair kept for the next call)
//   draw(srrd)  one draw of a built-in SRRDType with createSymRRD's default parameters, the
//               values of one block kept for the next calls of the same srrd
//   index(n)    uniform on {0, .., n - 1} (multiply-shift of 32 bits)
// With the Gaussian SRRDType's draws in coordinate order, normal() gives the built-in
// all-coordinate move's values (box_muller of the same blocks).
template <class R> struct UserRng {
    PhiloxCtx ph;
    uint32_t blk, iblk;
    uint32_t w[4];
    int nw;
    R spare;
    bool has_spare;
    R cache[4];
    int ncache, cache_srrd;
    const double *tape;
    int64_t *tpos;
    int64_t tlen;
    int *err;

    __device__ __forceinline__ double tape_next()
    {
        if (*tpos < tlen) { return tape[(*tpos)++]; }
        *err = 1;
        return 0.5;
    }
    __device__ __forceinline__ P4 next_block() { return ph.block(0, TAG_MOVE, blk++ & 0xfffu); }
    __device__ uint32_t bits()
    {
        if (tape) { return (uint32_t)tape_next(); }
        if (nw == 0) {
            const P4 q = next_block();
            w[0] = q.a;
            w[1] = q.b;
            w[2] = q.c;
            w[3] = q.d;
            nw = 4;
        }
        return w[4 - nw--];
    }
    __device__ R uniform()
    {
        if (tape) { return (R)tape_next(); }
        if constexpr (std::is_same<R, double>::value) {
            const uint32_t hi = bits(), lo = bits();
            return u01_d(hi, lo);
        } else {
            return u01_f(bits());
        }
    }
    __device__ R normal()
    {
        if (tape) { return (R)tape_next(); }
        if (has_spare) {
            has_spare = false;
            return spare;
        }
        R z0, z1;
        if constexpr (std::is_same<R, double>::value) {
            P4 q;
            q.a = bits();
            q.b = bits();
            q.c = bits();
            q.d = bits();
            box_muller_d(q, z0, z1);
        } else {
            const uint32_t a = bits(), b = bits();
            box_muller_f(a, b, z0, z1);
        }
        spare = z1;
        has_spare = true;
        return z0;
    }
    __device__ R draw(int srrd)
    {
        if (tape) { return (R)tape_next(); }
        if (ncache == 0 || cache_srrd != srrd) {
            move_draws_srrd<R>(next_block(), srrd, cache);
            ncache = Cpb<R>::v;
            cache_srrd = srrd;
        }
        return cache[Cpb<R>::v - ncache--];
    }
    __device__ int index(int n)
    {
        if (tape) {
            const int v = (int)tape_next();
            return v < 0 ? 0 : (v >= n ? n - 1 : v);
        }
        return (int)__umulhi(ph.block(0, TAG_INDEX, iblk++ & 0xfffu).a, (uint32_t)n);
    }
};

// What a dependent observable reads (DependentObservableInterface.hpp:24-53: registerDeps
// hands it pointers into the sampling functions and the earlier accumulators): for the
// handle's sampling function k, its proto values at the walker (protoold after the step; NULL
// for built-in kinds, whose protos are not kept) and the data its observationCallback prepared
// for this observation (SamplingFunctionInterface::prepareObservation, :59-62; NULL without
// one); and the values of the observables accumulated before this one in the same step, at
// their value offsets (the reference's rule: a dependent observable reads only earlier
// observables whose nskip divides its own).
template <class R> struct UserDeps {
    int npdf;
    int nproto[MCIG_MAXPDF];
    const R *proto[MCIG_MAXPDF];
    const R *prep[MCIG_MAXPDF];
    const R *obsvals;
};

template <class... P> struct PdfList {};
template <class... O> struct ObsList {};
template <class... M> struct MoveList {};

// optional members of a sampling function: observationCallback(args, x, protov, prep) with
// max_nprep prepared values; of an observable: observableFunction(args, x, out, deps)
template <class T, class R, class = void> struct HasObservationCallback : std::false_type {};
template <class T, class R>
struct HasObservationCallback<T, R,
                              std::void_t<decltype(T::observationCallback(std::declval<const UserArgs &>(),
                                                                          std::declval<const R *>(), std::declval<const R *>(),
                                                                          std::declval<R *>()))>> : std::true_type {};
template <class T, class R, class = void> struct HasObsDeps : std::false_type {};
template <class T, class R>
struct HasObsDeps<T, R,
                  std::void_t<decltype(T::observableFunction(std::declval<const UserArgs &>(), std::declval<const R *>(),
                                                             std::declval<R *>(), std::declval<const UserDeps<R> &>()))>>
    : std::true_type {};
template <class T, class = void> struct MaxNPrep { static constexpr int value = 0; };
template <class T> struct MaxNPrep<T, std::void_t<decltype(T::max_nprep)>> { static constexpr int value = T::max_nprep; };

// optional members of a trial move: proto values (max_nproto, nproto, protoFunction)
template <class T, class = void> struct MoveMaxNProto { static constexpr int value = 0; };
template <class T> struct MoveMaxNProto<T, std::void_t<decltype(T::max_nproto)>> { static constexpr int value = T::max_nproto; };
template <class T, class = void> struct HasMoveNProto : std::false_type {};
template <class T> struct HasMoveNProto<T, std::void_t<decltype(T::nproto(0))>> : std::true_type {};
template <class T, class R, class = void> struct HasMoveProto : std::false_type {};
template <class T, class R>
struct HasMoveProto<T, R,
                    std::void_t<decltype(T::protoFunction(std::declval<const UserArgs &>(), std::declval<const R *>(),
                                                          std::declval<R *>()))>> : std::true_type {};

template <class T, class R, class = void> struct HasUpdatedAcceptance : std::false_type {};
template <class T, class R>
struct HasUpdatedAcceptance<T, R,
                            std::void_t<decltype(T::updatedAcceptance(std::declval<const UserArgs &>(),
                                                                      std::declval<const UserWalker<R> &>(),
                                                                      std::declval<const R *>(), std::declval<R *>()))>>
    : std::true_type {};

constexpr int cmax() { return 1; }
template <class... T> constexpr int cmax(int a, T... b)
{
    const int r = cmax(b...);
    return a > r ? a : r;
}

// SamplingFunctionInterface::updatedAcceptance, or its default: every proto value anew
// (SamplingFunctionInterface.hpp:87-92)
template <class P, class R>
__device__ __forceinline__ R updated_or_full(const UserArgs &a, const UserWalker<R> &w, const R *po, R *pn)
{
    if constexpr (HasUpdatedAcceptance<P, R>::value) { return P::updatedAcceptance(a, w, po, pn); }
    else {
        P::protoFunction(a, w.xnew, pn);
        return P::acceptanceFunction(a, po, pn);
    }
}

template <class PL, class OL, class ML = MoveList<>> struct UserTable;

// dispatch from a runtime index to the k-th struct of each list
template <class... P, class... O, class... M> struct UserTable<PdfList<P...>, ObsList<O...>, MoveList<M...>> {
    static constexpr int npdf = (int)sizeof...(P);
    static constexpr int nobs = (int)sizeof...(O);
    static constexpr int nmove = (int)sizeof...(M);
    static constexpr int max_nproto = cmax(P::max_nproto...);
    static constexpr int max_nprep = cmax(MaxNPrep<P>::value...); // 1 when no sampling function prepares data
    static constexpr int move_max_nproto = cmax(MoveMaxNProto<M>::value...);
    static constexpr bool any_deps = (HasObsDeps<O, double>::value || ... || false);

    // trial moves, host side: -1 for k out of range
    template <class MM> static int move_nproto_one(int ndim)
    {
        if constexpr (HasMoveNProto<MM>::value) { return MM::nproto(ndim); }
        else { return 0; }
    }
    static int move_nproto(int k, int ndim)
    {
        int r = -1, i = 0;
        ((k == i++ ? (void)(r = move_nproto_one<M>(ndim)) : (void)0), ...);
        return r;
    }
    static int move_nstep(int k, const UserArgs &a)
    {
        int r = -1, i = 0;
        ((k == i++ ? (void)(r = M::nstep(a)) : (void)0), ...);
        return r;
    }
    static double move_step0(int k, const UserArgs &a, int t)
    {
        double r = 0.;
        int i = 0;
        ((k == i++ ? (void)(r = M::step0(a, t)) : (void)0), ...);
        return r;
    }
    static int move_step_index(int k, const UserArgs &a, int xidx)
    {
        int r = -1, i = 0;
        ((k == i++ ? (void)(r = M::step_index(a, xidx)) : (void)0), ...);
        return r;
    }
    static double move_change_rate(int k, const UserArgs &a)
    {
        double r = 0.;
        int i = 0;
        ((k == i++ ? (void)(r = M::change_rate(a)) : (void)0), ...);
        return r;
    }
    // trial moves, device side: ProtoFunctionInterface::initializeProtoValues and trialMove
    template <class MM, class R> __device__ static void move_proto_one(const UserArgs &a, const R *x, R *pv)
    {
        if constexpr (HasMoveProto<MM, R>::value) { MM::protoFunction(a, x, pv); }
    }
    template <class R> __device__ static void move_proto(int k, const UserArgs &a, const R *x, R *pv)
    {
        int i = 0;
        ((k == i++ ? move_proto_one<M, R>(a, x, pv) : (void)0), ...);
    }
    template <class R>
    __device__ static R move(int k, const UserArgs &a, UserMoveWalker<R> &w, const R *steps, UserRng<R> &rng, const R *po, R *pn)
    {
        R r = (R)1;
        int i = 0;
        ((k == i++ ? (void)(r = M::trialMove(a, w, steps, rng, po, pn)) : (void)0), ...);
        return r;
    }

    static int nproto(int k, int ndim)
    {
        int r = -1, i = 0;
        ((k == i++ ? (void)(r = P::nproto(ndim)) : (void)0), ...);
        return r;
    }
    static int nvals(int k, int ndim)
    {
        int r = -1, i = 0;
        ((k == i++ ? (void)(r = O::nobs(ndim)) : (void)0), ...);
        return r;
    }
    template <class R> __device__ static void proto(int k, const UserArgs &a, const R *x, R *pv)
    {
        int i = 0;
        ((k == i++ ? P::protoFunction(a, x, pv) : (void)0), ...);
    }
    template <class R> __device__ static R sampling(int k, const UserArgs &a, const R *pv)
    {
        R r = (R)0;
        int i = 0;
        ((k == i++ ? (void)(r = P::samplingFunction(a, pv)) : (void)0), ...);
        return r;
    }
    // computeAcceptance (SamplingFunctionInterface.hpp:49-57): partial moves through
    // updatedAcceptance, all-moves through protoFunction + acceptanceFunction
    template <class R>
    __device__ static R accept(int k, const UserArgs &a, const UserWalker<R> &w, bool partial, const R *po, R *pn)
    {
        R r = (R)0;
        int i = 0;
        ((k == i++ ? (void)(r = partial ? updated_or_full<P, R>(a, w, po, pn)
                                        : (P::protoFunction(a, w.xnew, pn), P::acceptanceFunction(a, po, pn)))
                   : (void)0),
         ...);
        return r;
    }
    template <class R> __device__ static void observe(int k, const UserArgs &a, const R *x, R *out)
    {
        int i = 0;
        ((k == i++ ? O::observableFunction(a, x, out) : (void)0), ...);
    }
    // observableFunction with the dependencies where the observable takes them
    template <class R> __device__ static void observe_deps(int k, const UserArgs &a, const R *x, R *out, const UserDeps<R> &d)
    {
        int i = 0;
        ((k == i++ ? observe_one<O, R>(a, x, out, d) : (void)0), ...);
    }
    template <class OO, class R> __device__ static void observe_one(const UserArgs &a, const R *x, R *out, const UserDeps<R> &d)
    {
        if constexpr (HasObsDeps<OO, R>::value) { OO::observableFunction(a, x, out, d); }
        else { OO::observableFunction(a, x, out); }
    }
    // SamplingFunctionInterface::prepareObservation (:59-62): observationCallback(x, protoold);
    // false for a sampling function without one
    template <class R> __device__ static bool prepare(int k, const UserArgs &a, const R *x, const R *pv, R *prep)
    {
        bool has = false;
        int i = 0;
        ((k == i++ ? (void)(has = prepare_one<P, R>(a, x, pv, prep)) : (void)0), ...);
        return has;
    }
    template <class PP, class R> __device__ static bool prepare_one(const UserArgs &a, const R *x, const R *pv, R *prep)
    {
        if constexpr (HasObservationCallback<PP, R>::value) {
            PP::observationCallback(a, x, pv, prep);
            return true;
        } else {
            return false;
        }
    }
};

// the built-in kernels: no user functors
using NoPlugin = UserTable<PdfList<>, ObsList<>, MoveList<>>;

} // namespace mcig
