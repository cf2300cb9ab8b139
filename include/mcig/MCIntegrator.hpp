// mcig/MCIntegrator.hpp -- C++ host facade of the GB300 integrator.
//
// mcig::MCI mirrors the reference's mci::MCI (include/mci/MCIntegrator.hpp:93-225
// of DCM-UPB/MCIntegratorPlusPlus) method by method over the C ABI of
// include/mcig.h, and throws the reference's exception types
// (std::invalid_argument, std::domain_error, std::runtime_error).  Sampling
// functions and observables are device functor descriptors (kind + parameters)
// built with the factory functions below, whose names follow the classes they
// reproduce (test/common/TestMCIFunctions.hpp).  One MCI object holds `nchains`
// chains on the GPU; integrate() combines them as MPIMCI combines ranks.
//
// Header-only; link with libmcigpu.so.
#ifndef MCIG_MCINTEGRATOR_HPP
#define MCIG_MCINTEGRATOR_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../mcig.h"

namespace mcig
{
enum class MoveType { All = MCIG_MOVE_ALL, Vec = MCIG_MOVE_VEC, MultiStep = MCIG_MOVE_MULTISTEP };
enum class SRRDType {
    Uniform = MCIG_SRRD_UNIFORM, Gaussian, Student, Cauchy, Exponential, Gamma, Weibull, Lognormal, Chisq, Fisher
};
enum class EstimatorType {
    Noop = MCIG_EST_NOOP, Uncorrelated, Correlated, FCBlocker, MJBlocker
};
enum class Precision { FP64 = MCIG_PREC_FP64, FP32 = MCIG_PREC_FP32, FP32Acc64 = MCIG_PREC_FP32_ACC64 };

// device functor descriptor (include/mcig_types.h kinds)
struct Functor {
    int kind;
    std::vector<double> params;
};
using SamplingFunction = Functor;
using Observable = Functor;

// sampling functions
inline SamplingFunction ThreeDimGaussianPDF() { return {MCIG_PDF_GAUSS_SUM, {}}; }
inline SamplingFunction Gauss() { return {MCIG_PDF_GAUSS, {}}; }
inline SamplingFunction ExpNDPDF() { return {MCIG_PDF_EXP, {}}; }
inline SamplingFunction GaussPrecision(const std::vector<double> &P /* ndim*ndim, row-major */) { return {MCIG_PDF_GAUSS_PREC, P}; }
inline SamplingFunction GaussBlock(int b0, int b1, double width) { return {MCIG_PDF_GAUSS_BLOCK, {double(b0), double(b1), width}}; }
// [ncomp, w[ncomp], m[ncomp*ndim], s[ncomp*ndim]]
inline SamplingFunction GaussMixture(const std::vector<double> &params) { return {MCIG_PDF_GAUSS_MIX, params}; }

// observables
inline Observable X2Sum() { return {MCIG_OBS_X2SUM, {}}; }
inline Observable XND() { return {MCIG_OBS_XND, {}}; }
inline Observable X2() { return {MCIG_OBS_X2, {}}; }
inline Observable XSquared() { return {MCIG_OBS_X2MEAN, {}}; }
inline Observable Constval(double v = 1.3) { return {MCIG_OBS_CONST, {v}}; }
inline Observable Polynom() { return {MCIG_OBS_POLYNOM, {}}; }
inline Observable GaussXSquared() { return {MCIG_OBS_GAUSSX2, {}}; }
inline Observable XI(int i) { return {MCIG_OBS_XI, {double(i)}}; }
// log of the product of the sampling functions at the walker: an observable that depends on them
inline Observable LogPDF() { return {MCIG_OBS_LOGPDF, {}}; }
inline Observable X2Blocks(const std::vector<int> &bounds /* b_0 < ... < b_nb */)
{
    Observable o{MCIG_OBS_X2BLOCK, {double(bounds.size() - 1)}};
    for (int b : bounds) { o.params.push_back(double(b)); }
    return o;
}

namespace detail
{
inline void check(int rc)
{
    if (rc == MCIG_OK) { return; }
    const std::string msg = mcig_last_error();
    switch (rc) {
    case MCIG_ERR_INVALID_ARGUMENT: throw std::invalid_argument(msg);
    case MCIG_ERR_DOMAIN: throw std::domain_error(msg);
    default: throw std::runtime_error(msg);
    }
}
inline const double *ptr(const std::vector<double> &v) { return v.empty() ? nullptr : v.data(); }
} // namespace detail

// a trial move of a plugin (TrialMoveInterface as a device struct): its index in the
// plugin's move list and the parameters handed to it
struct UserMove
{
    int k;
    std::vector<double> params;
};

// user sampling functions, observables and trial moves compiled for the device
// (mcig/plugin.cuh): the loaded library; its k-th functors are pdf(k, params), obs(k, params)
// and move(k, params).  It must outlive every MCI that uses it.
class Plugin
{
private:
    mcig_plugin *_p = nullptr;

public:
    explicit Plugin(const std::string &path) { detail::check(mcig_plugin_load(path.c_str(), &_p)); }
    ~Plugin() { mcig_plugin_unload(_p); }
    Plugin(const Plugin &) = delete;
    Plugin &operator=(const Plugin &) = delete;
    const mcig_plugin *handle() const { return _p; }
    static SamplingFunction pdf(int k, std::vector<double> params = {}) { return {MCIG_PDF_USER + k, std::move(params)}; }
    static Observable obs(int k, std::vector<double> params = {}) { return {MCIG_OBS_USER + k, std::move(params)}; }
    static UserMove move(int k, std::vector<double> params = {}) { return {k, std::move(params)}; }
};

class MCI
{
private:
    mcig_mci *_h = nullptr;
    int _ndim;
    int64_t _nchains;
    double _target = 0.5;
    int _nfind = -50;
    int64_t _ndecorr = -10000;

public:
    explicit MCI(int ndim, int64_t nchains = 1, int device = 0, Precision prec = Precision::FP64):
            _ndim(ndim), _nchains(nchains)
    {
        detail::check(mcig_create(ndim, nchains, device, static_cast<int>(prec), &_h));
    }
    ~MCI() { mcig_destroy(_h); }
    MCI(const MCI &) = delete;
    MCI &operator=(const MCI &) = delete;
    MCI(MCI &&o) noexcept: _h(o._h), _ndim(o._ndim), _nchains(o._nchains) { o._h = nullptr; }

    mcig_mci *handle() const { return _h; }

    // --- setters
    void setPlugin(const Plugin *pl) { detail::check(mcig_set_plugin(_h, pl ? pl->handle() : nullptr)); }
    void setSeed(uint64_t seed) { detail::check(mcig_set_seed(_h, seed)); }
    // file output of chain 0 during the main sampling (MCIntegrator.hpp storeObservablesOnFile et al.)
    void storeObservablesOnFile(const std::string &path, int freq) { detail::check(mcig_store_observables_on_file(_h, path.c_str(), freq)); }
    void clearObservableFile() { detail::check(mcig_clear_observable_file(_h)); }
    void storeWalkerPositionsOnFile(const std::string &path, int freq) { detail::check(mcig_store_walker_positions_on_file(_h, path.c_str(), freq)); }
    void clearWalkerFile() { detail::check(mcig_clear_walker_file(_h)); }
    void setX(int i, double val)
    {
        std::vector<double> x = getXAll();
        for (int64_t c = 0; c < _nchains; ++c) { x[c * _ndim + i] = val; }
        detail::check(mcig_set_x(_h, x.data(), _nchains));
    }
    void setX(const double x[]) { detail::check(mcig_set_x(_h, x, 1)); }                    // same x for every chain
    void setXAll(const double x[] /* [nchains][ndim] */) { detail::check(mcig_set_x(_h, x, _nchains)); }
    void centerX() { detail::check(mcig_center_x(_h)); }
    void setMRT2Step(double s) { detail::check(mcig_set_mrt2step(_h, s)); }
    void setMRT2Step(int i, double s) { detail::check(mcig_set_mrt2step_i(_h, i, s)); }
    void setMRT2Step(const double s[])
    {
        int n = 0;
        detail::check(mcig_get_nstepsizes(_h, &n));
        for (int i = 0; i < n; ++i) { setMRT2Step(i, s[i]); }
    }
    void setTargetAcceptanceRate(double r) { _target = r; detail::check(mcig_set_target_acceptance_rate(_h, r)); }
    void setNfindMRT2Iterations(int n) { _nfind = n; detail::check(mcig_set_nfind_mrt2_iterations(_h, n)); }
    void setNdecorrelationSteps(int64_t n) { _ndecorr = n; detail::check(mcig_set_ndecorrelation_steps(_h, n)); }
    void setPrecision(Precision p) { detail::check(mcig_set_precision(_h, static_cast<int>(p))); }
    // device tuning without a counterpart in mci::MCI (results unchanged, include/mcig.h):
    // kernel choice 0 automatic / 1 general / 2 register-resident, the calibration's tail on
    // four lanes per chain (default on), the three phases in one launch (default off), lanes
    // per chain of the multi-lane kernels (0 automatic, 1, 2, 4, 8)
    void setKernel(int policy) { detail::check(mcig_set_kernel(_h, policy)); }
    void setCalibrationSplit(bool on) { detail::check(mcig_set_calibration_split(_h, on ? 1 : 0)); }
    void setPhaseFusion(bool on) { detail::check(mcig_set_phase_fusion(_h, on ? 1 : 0)); }
    void setLanes(int lanes_per_chain) { detail::check(mcig_set_lanes(_h, lanes_per_chain)); }

    // --- domain
    void setIRange(double lb, double ub)
    {
        std::vector<double> l(_ndim, lb), u(_ndim, ub);
        detail::check(mcig_set_irange(_h, l.data(), u.data()));
    }
    void setIRange(const double lb[], const double ub[]) { detail::check(mcig_set_irange(_h, lb, ub)); }
    void resetDomain() { detail::check(mcig_reset_domain(_h)); }

    // --- trial moves
    void setTrialMove(MoveType m) { detail::check(mcig_set_trial_move(_h, static_cast<int>(m), MCIG_SRRD_UNIFORM, 1, 1, nullptr)); }
    // MCI::setTrialMove(std::unique_ptr<TrialMoveInterface>): a plugin's move (setPlugin first)
    void setTrialMove(const UserMove &m) { detail::check(mcig_set_user_move(_h, m.k, detail::ptr(m.params), (int)m.params.size())); }
    void setTrialMove(SRRDType srrd, int veclen = 0, int ntypes = 1, int typeEnds[] = nullptr)
    {
        detail::check(mcig_set_trial_move(_h, veclen > 0 ? MCIG_MOVE_VEC : MCIG_MOVE_ALL, static_cast<int>(srrd),
                                          veclen, ntypes, typeEnds));
    }
    // MultiStepMove(ndim, nsteps) with sub-move SRRDVecMove(ndim/veclen, veclen, step) and sub-pdfs
    void setMultiStepMove(int nsteps, SRRDType sub, int sub_veclen, double sub_step,
                          const std::vector<SamplingFunction> &subpdfs)
    {
        detail::check(mcig_set_multistep_move(_h, nsteps, static_cast<int>(sub), sub_veclen, sub_step));
        for (auto &f : subpdfs) {
            detail::check(mcig_multistep_add_pdf(_h, f.kind, detail::ptr(f.params), (int)f.params.size()));
        }
    }

    // --- observables
    void addObservable(const Observable &o, int blocksize, int nskip, bool flag_equil, bool flag_correlated)
    {
        blocksize = blocksize < 0 ? 0 : blocksize;
        const bool flag_error = blocksize > 0;
        if (flag_correlated && !flag_error) {
            throw std::invalid_argument("[selectEstimatorType] Error calculation is set off, but correlated error estimation is set on.");
        }
        const EstimatorType e = flag_correlated ? EstimatorType::Correlated
                                                : (flag_error ? EstimatorType::Uncorrelated : EstimatorType::Noop);
        addObservable(o, blocksize, nskip, flag_equil, e);
    }
    void addObservable(const Observable &o, int blocksize = 1, int nskip = 1)
    {
        addObservable(o, blocksize, nskip, blocksize > 0, blocksize == 1);
    }
    void addObservable(const Observable &o, int blocksize, int nskip, bool flag_equil, EstimatorType e)
    {
        detail::check(mcig_add_observable(_h, o.kind, detail::ptr(o.params), (int)o.params.size(), blocksize, nskip,
                                          flag_equil ? 1 : 0, static_cast<int>(e)));
    }
    void popObservable() { detail::check(mcig_pop_observable(_h)); }
    void clearObservables() { detail::check(mcig_clear_observables(_h)); }
    void setFullStorage(int bits) { detail::check(mcig_set_full_storage(_h, bits)); }

    // --- sampling functions
    void addSamplingFunction(const SamplingFunction &f)
    {
        detail::check(mcig_add_sampling_function(_h, f.kind, detail::ptr(f.params), (int)f.params.size()));
    }
    void popSamplingFunction() { detail::check(mcig_pop_sampling_function(_h)); }
    void clearSamplingFunctions() { detail::check(mcig_clear_sampling_functions(_h)); }

    // --- getters
    int getNDim() const { return _ndim; }
    int64_t getNChains() const { return _nchains; }
    std::vector<double> getXAll() const
    {
        std::vector<double> x((size_t)_nchains * _ndim);
        detail::check(mcig_get_x(_h, x.data()));
        return x;
    }
    double getX(int i, int64_t chain = 0) const { return getXAll()[chain * _ndim + i]; }
    double getMRT2Step(int i) const
    {
        double v = 0.;
        detail::check(mcig_get_mrt2step(_h, 0, i, &v));
        return v;
    }
    double getTargetAcceptanceRate() const { return _target; }
    double getAcceptanceRate() const
    {
        double r = 0.;
        detail::check(mcig_get_acceptance_rate(_h, &r));
        return r;
    }
    int getNfindMRT2Iterations() const { return _nfind; }
    int64_t getNdecorrelationSteps() const { return _ndecorr; }
    int getNPDF() const
    {
        int n = 0;
        detail::check(mcig_get_npdf(_h, &n));
        return n;
    }
    int getNObs() const
    {
        int n = 0;
        detail::check(mcig_get_nobs(_h, &n));
        return n;
    }
    int getNObsDim() const
    {
        int n = 0;
        detail::check(mcig_get_nobsdim(_h, &n));
        return n;
    }

    // --- integrate (MCIntegrator.hpp:225)
    void integrate(int64_t Nmc, double average[], double error[], bool doFindMRT2step = true, bool doDecorrelation = true)
    {
        detail::check(mcig_integrate(_h, Nmc, average, error, doFindMRT2step ? 1 : 0, doDecorrelation ? 1 : 0));
    }
};
} // namespace mcig

#endif
