// mcig/plugin.cuh -- user sampling functions and observables for the GB300 integrator.
//
// The reference integrates user code derived from mci::SamplingFunctionInterface and
// mci::ObservableFunctionInterface (include/mci/SamplingFunctionInterface.hpp:37-104,
// include/mci/ObservableFunctionInterface.hpp:24-60).  Here the same functions are static
// members of structs compiled for the device; a plugin is a shared library that builds the
// general sampling kernel over a list of them:
//
//   #include <mcig/plugin.cuh>
//
//   struct MyGauss {                                     // exp(-sum_i x_i^2), one proto per index
//       static constexpr int max_nproto = 64;
//       static int nproto(int ndim) { return ndim; }
//       template <class R> __device__ static void protoFunction(const mcig::UserArgs &a, const R *in, R *pv)
//       { for (int i = 0; i < a.ndim; ++i) { pv[i] = in[i] * in[i]; } }
//       template <class R> __device__ static R samplingFunction(const mcig::UserArgs &a, const R *pv) { ... }
//       template <class R> __device__ static R acceptanceFunction(const mcig::UserArgs &a, const R *po, const R *pn) { ... }
//       // optional, for moves that change a few coordinates (changed: w.lo .. w.lo + w.nchanged - 1)
//       template <class R> __device__ static R updatedAcceptance(const mcig::UserArgs &a, const mcig::UserWalker<R> &w,
//                                                                 const R *po, R *pn) { ... }
//   };
//   struct MyObs {
//       static int nobs(int ndim) { return 1; }
//       template <class R> __device__ static void observableFunction(const mcig::UserArgs &a, const R *in, R *out) { ... }
//   };
//   using MyPdfs = mcig::PdfList<MyGauss>;
//   using MyObss = mcig::ObsList<MyObs>;
//   MCIG_PLUGIN(MyPdfs, MyObss)
//
// With user trial moves (TrialMoveInterface, include/mci/TrialMoveInterface.hpp:18-75):
//
//   struct MyGaussMove {                                 // x' = x + s z, z ~ N(0, I), one step size
//       static int nstep(const mcig::UserArgs &) { return 1; }
//       static double step0(const mcig::UserArgs &, int) { return 0.05; }
//       static int step_index(const mcig::UserArgs &, int) { return 0; }
//       static double change_rate(const mcig::UserArgs &) { return 1.; }
//       template <class R>
//       __device__ static R trialMove(const mcig::UserArgs &a, mcig::UserMoveWalker<R> &w, const R *steps,
//                                     mcig::UserRng<R> &rng, const R *, R *)
//       {
//           for (int i = 0; i < a.ndim; ++i) { w.xnew[i] = w.xold[i] + steps[0] * rng.normal(); }
//           w.nchanged = a.ndim;
//           return (R)1;                                 // symmetric move
//       }
//   };
//   MCIG_PLUGIN_MOVES(MyPdfs, MyObss, mcig::MoveList<MyGaussMove>)
//
// and mcig_set_user_move(handle, k, params, nparams) installs the k-th move.
//
// Build (mcintegratorplusplus_gb300.build.build_plugin does this): the source compiled twice,
// once with -DMCIG_PLUGIN_PART=1 -fmad=false (double path, the reference's operation order)
// and once with -DMCIG_PLUGIN_PART=2 (float path), both objects linked with -shared; one
// compilation without MCIG_PLUGIN_PART builds both paths with the same flags.  Include paths:
// this directory's parent and mcintegratorplusplus_gb300/csrc.
//
// Use: mcig_plugin_load(path), mcig_set_plugin(handle, plugin), then the kinds
// MCIG_PDF_USER + k and MCIG_OBS_USER + k with the functor's parameters (UserArgs::params).
// R is double in the MCIG_PREC_FP64 path and float in the float paths; the float Metropolis
// test takes the log of acceptanceFunction's ratio.
#ifndef MCIG_PLUGIN_CUH
#define MCIG_PLUGIN_CUH

#include "mcig_generic.cuh"
#include "mcig_launchers.h"

namespace mcig
{
namespace plugin_detail
{
// launch, then the launch's own error code from this library's CUDA runtime
template <class U, class R, int RNG, bool KAHAN>
int launch(const KParams &p, int movetype, int grid, int block, size_t smem, cudaStream_t st)
{
    auto k = mcig_generic_kernel<R, RNG, KAHAN, U>;
    if (smem > 48 * 1024) { cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); }
    k<<<grid, block, smem, st>>>(p, movetype);
    return (int)cudaGetLastError();
}
} // namespace plugin_detail
} // namespace mcig

#define MCIG_PLUGIN_F32_(TABLE)                                                                                   \
    extern "C" mcig_plugin_launch_fn mcig_plugin_launcher_f32(int precision)                                      \
    {                                                                                                             \
        return precision == MCIG_PREC_FP32 ? mcig::plugin_detail::launch<TABLE, float, RNG_PHILOX, true>          \
                                           : mcig::plugin_detail::launch<TABLE, float, RNG_PHILOX, false>;        \
    }

#define MCIG_PLUGIN_MAIN_(TABLE)                                                                                  \
    extern "C" int mcig_plugin_abi(void) { return MCIG_PLUGIN_ABI; }                                              \
    extern "C" int mcig_plugin_kparams_size(void) { return (int)sizeof(KParams); }                               \
    extern "C" int mcig_plugin_npdf(void) { return TABLE::npdf; }                                                 \
    extern "C" int mcig_plugin_nobs(void) { return TABLE::nobs; }                                                 \
    extern "C" int mcig_plugin_pdf_nproto(int k, int ndim)                                                        \
    {                                                                                                             \
        const int n = TABLE::nproto(k, ndim);                                                                     \
        return (n < 0 || n > TABLE::max_nproto) ? -1 : n;                                                         \
    }                                                                                                             \
    extern "C" int mcig_plugin_obs_nvals(int k, int ndim) { return TABLE::nvals(k, ndim); }                      \
    extern "C" int mcig_plugin_nmove(void) { return TABLE::nmove; }                                               \
    extern "C" int mcig_plugin_move_info(int k, int ndim, const double *params, int nparams, int *nproto,         \
                                         int *nstep, double *change_rate)                                         \
    {                                                                                                             \
        if (k < 0 || k >= TABLE::nmove) { return -1; }                                                           \
        const mcig::UserArgs a{ndim, params, nparams};                                                            \
        const int np = TABLE::move_nproto(k, ndim);                                                               \
        *nproto = (np < 0 || np > TABLE::move_max_nproto) ? -1 : np;                                              \
        *nstep = TABLE::move_nstep(k, a);                                                                         \
        *change_rate = TABLE::move_change_rate(k, a);                                                             \
        return 0;                                                                                                 \
    }                                                                                                             \
    extern "C" int mcig_plugin_move_steps(int k, int ndim, const double *params, int nparams, int nstep,          \
                                          double *step0, int *stepidx)                                            \
    {                                                                                                             \
        if (k < 0 || k >= TABLE::nmove) { return -1; }                                                           \
        const mcig::UserArgs a{ndim, params, nparams};                                                            \
        for (int t = 0; t < nstep; ++t) { step0[t] = TABLE::move_step0(k, a, t); }                                \
        for (int i = 0; i < ndim; ++i) { stepidx[i] = TABLE::move_step_index(k, a, i); }                          \
        return 0;                                                                                                 \
    }                                                                                                             \
    extern "C" mcig_plugin_launch_fn mcig_plugin_launcher_f32(int precision);                                     \
    extern "C" mcig_plugin_launch_fn mcig_plugin_launcher(int precision, int rng)                                 \
    {                                                                                                             \
        if (precision == MCIG_PREC_FP64) {                                                                        \
            return rng == RNG_TAPE ? mcig::plugin_detail::launch<TABLE, double, RNG_TAPE, false>                  \
                                   : mcig::plugin_detail::launch<TABLE, double, RNG_PHILOX, false>;               \
        }                                                                                                         \
        return rng == RNG_PHILOX ? mcig_plugin_launcher_f32(precision) : nullptr;                                 \
    }

#if !defined(MCIG_PLUGIN_PART)
#define MCIG_PLUGIN_MOVES(PDFS, OBSS, MOVES)                                                                      \
    using mcig_plugin_table_ = mcig::UserTable<PDFS, OBSS, MOVES>;                                                \
    MCIG_PLUGIN_MAIN_(mcig_plugin_table_)                                                                         \
    MCIG_PLUGIN_F32_(mcig_plugin_table_)
#elif MCIG_PLUGIN_PART == 1
#define MCIG_PLUGIN_MOVES(PDFS, OBSS, MOVES)                                                                      \
    using mcig_plugin_table_ = mcig::UserTable<PDFS, OBSS, MOVES>;                                                \
    MCIG_PLUGIN_MAIN_(mcig_plugin_table_)
#else
#define MCIG_PLUGIN_MOVES(PDFS, OBSS, MOVES)                                                                      \
    using mcig_plugin_table_ = mcig::UserTable<PDFS, OBSS, MOVES>;                                                \
    MCIG_PLUGIN_F32_(mcig_plugin_table_)
#endif
#define MCIG_PLUGIN(PDFS, OBSS) MCIG_PLUGIN_MOVES(PDFS, OBSS, mcig::MoveList<>)

#endif
