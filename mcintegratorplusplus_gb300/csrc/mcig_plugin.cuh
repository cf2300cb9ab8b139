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

// WalkerState (include/mci/WalkerState.hpp) of a partial move: xold/xnew, and the changed
// coordinates lo, lo + 1, ..., lo + nchanged - 1 (the ascending changedIdx of the reference)
template <class R> struct UserWalker {
    const R *xold;
    const R *xnew;
    int nchanged;
    int lo;
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

template <class PL, class OL> struct UserTable;

// dispatch from a runtime index to the k-th struct of each list
template <class... P, class... O> struct UserTable<PdfList<P...>, ObsList<O...>> {
    static constexpr int npdf = (int)sizeof...(P);
    static constexpr int nobs = (int)sizeof...(O);
    static constexpr int max_nproto = cmax(P::max_nproto...);
    static constexpr int max_nprep = cmax(MaxNPrep<P>::value...); // 1 when no sampling function prepares data
    static constexpr bool any_deps = (HasObsDeps<O, double>::value || ... || false);

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
using NoPlugin = UserTable<PdfList<>, ObsList<>>;

} // namespace mcig
