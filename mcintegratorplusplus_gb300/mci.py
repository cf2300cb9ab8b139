"""Python mirror of the reference's integrator facade ``mci::MCI``
(include/mci/MCIntegrator.hpp:93-225 of DCM-UPB/MCIntegratorPlusPlus) over the C
ABI of libmcigpu.so (include/mcig.h).

Method names follow the reference (setSeed, addSamplingFunction,
addObservable, integrate, ...); snake_case aliases exist for the shared test
configuration.  Exceptions follow the reference's: std::invalid_argument ->
ValueError, std::domain_error -> DomainError, std::runtime_error -> RuntimeError.

Differences from the reference, by design of the device path:
  * one object holds `nchains` independent chains (one per GPU thread);
    integrate() combines them with the MPIMCI formula (src/MPIMCI.cpp:85-92);
  * sampling functions and observables are device functors chosen by kind
    (include/mcig_types.h) instead of virtual C++ objects; user functors are
    structs compiled into a plugin (include/mcig/plugin.cuh, Plugin below);
  * the seed keys a Philox4x32-10 stream instead of std::mt19937_64 (replay
    mode consumes the reference's recorded draws instead).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import P_double, P_int, P_int64, P_uint8, P_uint32

OK, ERR_INVALID, ERR_DOMAIN, ERR_RUNTIME, ERR_CUDA, ERR_UNSUPPORTED, ERR_TIMEOUT = range(7)

# enums of include/mcig_types.h
MOVE_ALL, MOVE_VEC, MOVE_MULTISTEP = 0, 1, 2
SRRD_UNIFORM, SRRD_GAUSSIAN, SRRD_STUDENT, SRRD_CAUCHY, SRRD_EXPONENTIAL, SRRD_GAMMA, SRRD_WEIBULL, \
    SRRD_LOGNORMAL, SRRD_CHISQ, SRRD_FISHER = range(10)
EST_NOOP, EST_UNCORRELATED, EST_CORRELATED, EST_FCBLOCKER, EST_MJBLOCKER = range(5)
PDF_GAUSS_SUM, PDF_GAUSS, PDF_EXP, PDF_GAUSS_PREC, PDF_GAUSS_BLOCK, PDF_GAUSS_MIX = range(6)
OBS_X2SUM, OBS_XND, OBS_X2, OBS_X2MEAN, OBS_CONST, OBS_POLYNOM, OBS_X2BLOCK, OBS_GAUSSX2, OBS_XI, OBS_LOGPDF = range(10)
PREC_FP64, PREC_FP32, PREC_FP32_ACC64 = range(3)
PDF_USER, OBS_USER = 100, 100  # + k: the k-th sampling function / observable of the handle's plugin


class DomainError(ValueError):
    """std::domain_error of the reference."""


class CudaError(RuntimeError):
    pass


def _raise(rc):
    if rc == OK:
        return
    msg = _lib.load().mcig_last_error().decode()
    if rc == ERR_INVALID:
        raise ValueError(msg)
    if rc == ERR_DOMAIN:
        raise DomainError(msg)
    if rc == ERR_RUNTIME:
        raise RuntimeError(msg)
    if rc == ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if rc == ERR_TIMEOUT:
        raise TimeoutError(msg)
    raise CudaError(msg)


def _dp(a):
    return a.ctypes.data_as(P_double)


def _params(params):
    p = np.ascontiguousarray(np.asarray(params if params is not None else (), dtype=np.float64).ravel())
    if p.size == 0:
        p = np.zeros(1)
        return p, 0
    return p, int(p.size)


class MCI:
    """mci::MCI on the GPU: `nchains` chains of dimension `ndim`."""

    def __init__(self, ndim, nchains=1, device=0, precision=PREC_FP64):
        self.L = _lib.load()
        self.ndim = int(ndim)
        self.nchains = int(nchains)
        h = ctypes.c_void_p()
        _raise(self.L.mcig_create(self.ndim, self.nchains, int(device), int(precision), ctypes.byref(h)))
        self._h = h
        self._tape = None

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.L.mcig_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setPlugin(self, plugin):
        """Attach a Plugin whose kinds PDF_USER + k / OBS_USER + k this MCI may use (None detaches)."""
        _raise(self.L.mcig_set_plugin(self._h, plugin._h if plugin is not None else None))
        self._plugin = plugin  # kept alive while the handle may use it

    # --- setters (MCIntegrator.hpp:96-123)
    def setSeed(self, seed):
        _raise(self.L.mcig_set_seed(self._h, ctypes.c_uint64(int(seed) & ((1 << 64) - 1))))

    def setKernel(self, policy):
        """0 automatic, 1 general kernel, 2 register-resident float kernel."""
        _raise(self.L.mcig_set_kernel(self._h, int(policy)))

    def setPhaseFusion(self, on=True):
        """Calibration, burn-in and sampling in one register-resident launch where it applies (default off: slower when a few chains calibrate long)."""
        _raise(self.L.mcig_set_phase_fusion(self._h, int(bool(on))))

    def setCalibrationSplit(self, on=True):
        """Calibration's tail on 4 lanes per chain where it applies (default on; same results)."""
        _raise(self.L.mcig_set_calibration_split(self._h, int(bool(on))))

    def setLanes(self, lpc):
        """Lanes per chain of the multi-lane kernels: 0 automatic (two lanes where they serve the
        configuration, there are at most 32,768 chains and an observable other than x or x.x),
        1 one lane, 2 (one exp(-x.x) or
        precision-matrix sampling function in 9..16 coordinates), 4 or 8 (one mixture in 17..32
        coordinates)."""
        _raise(self.L.mcig_set_lanes(self._h, int(lpc)))

    def setSamplingChunks(self, n):
        """Main sampling in n launches with the Full-sample estimator overlapped (1: one launch)."""
        _raise(self.L.mcig_set_sampling_chunks(self._h, int(n)))

    def setFP64Decision(self, mode=1):
        """Metropolis decision certified in double near the float threshold (1), on every step (2), off (0)."""
        _raise(self.L.mcig_set_fp64_decision(self._h, int(mode)))

    def getDecisionStats(self):
        """(steps tested in double, float decisions reversed, largest reversed float margin) of the last integrate."""
        a, b, m = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
        _raise(self.L.mcig_get_decision_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(m)))
        return a.value, b.value, m.value

    def setPrecision(self, precision):
        _raise(self.L.mcig_set_precision(self._h, int(precision)))

    def setX(self, x):
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
        n = 1 if x.ndim == 1 else x.shape[0]
        if x.size != n * self.ndim:
            raise ValueError("setX: expected %d values per chain" % self.ndim)
        _raise(self.L.mcig_set_x(self._h, _dp(x), n))

    def getX(self):
        x = np.zeros((self.nchains, self.ndim))
        _raise(self.L.mcig_get_x(self._h, _dp(x)))
        return x

    def centerX(self):
        _raise(self.L.mcig_center_x(self._h))

    def setMRT2Step(self, step, i=None):
        if i is None:
            _raise(self.L.mcig_set_mrt2step(self._h, float(step)))
        else:
            _raise(self.L.mcig_set_mrt2step_i(self._h, int(i), float(step)))

    def getMRT2Step(self, i=0, chain=0):
        v = ctypes.c_double()
        _raise(self.L.mcig_get_mrt2step(self._h, int(chain), int(i), ctypes.byref(v)))
        return v.value

    def getMRT2Steps(self):
        n = ctypes.c_int()
        _raise(self.L.mcig_get_nstepsizes(self._h, ctypes.byref(n)))
        out = np.zeros((self.nchains, n.value))
        _raise(self.L.mcig_get_mrt2steps(self._h, _dp(out)))
        return out

    def setTargetAcceptanceRate(self, rate):
        _raise(self.L.mcig_set_target_acceptance_rate(self._h, float(rate)))

    def setNfindMRT2Iterations(self, n):
        _raise(self.L.mcig_set_nfind_mrt2_iterations(self._h, int(n)))

    def setNdecorrelationSteps(self, n):
        _raise(self.L.mcig_set_ndecorrelation_steps(self._h, int(n)))

    # --- moves (MCIntegrator.hpp:139-146)
    def setTrialMove(self, movetype=MOVE_ALL, srrd=SRRD_UNIFORM, veclen=0, ntypes=1, typeEnds=None):
        te = None
        if typeEnds is not None:
            te = (ctypes.c_int * len(typeEnds))(*[int(v) for v in typeEnds])
        _raise(self.L.mcig_set_trial_move(self._h, int(movetype), int(srrd), int(veclen), int(ntypes), te))

    def setUserMove(self, k, params=None):
        """The attached plugin's k-th trial move as this MCI's move (MCI::setTrialMove with a
        TrialMoveInterface object); params are handed to the move."""
        p, n = _params(params)
        _raise(self.L.mcig_set_user_move(self._h, int(k), _dp(p), n))

    def setMultiStepMove(self, nsteps, sub_srrd=SRRD_UNIFORM, sub_veclen=1, sub_step=0.05):
        _raise(self.L.mcig_set_multistep_move(self._h, int(nsteps), int(sub_srrd), int(sub_veclen), float(sub_step)))

    def addMultiStepSamplingFunction(self, kind, params=None):
        p, n = _params(params)
        _raise(self.L.mcig_multistep_add_pdf(self._h, int(kind), _dp(p), n))

    # --- sampling functions (MCIntegrator.hpp:181-184)
    def addSamplingFunction(self, kind, params=None):
        p, n = _params(params)
        _raise(self.L.mcig_add_sampling_function(self._h, int(kind), _dp(p), n))

    def popSamplingFunction(self):
        _raise(self.L.mcig_pop_sampling_function(self._h))

    def clearSamplingFunctions(self):
        _raise(self.L.mcig_clear_sampling_functions(self._h))

    def getNPDF(self):
        n = ctypes.c_int()
        _raise(self.L.mcig_get_npdf(self._h, ctypes.byref(n)))
        return n.value

    # --- observables (MCIntegrator.hpp:150-177)
    def addObservable(self, kind, params=None, blocksize=1, nskip=1, flag_equil=None, estimator=None):
        """addObservable(obs, blocksize, nskip[, flag_equil, EstimatorType or flag_correlated])."""
        p, n = _params(params)
        if flag_equil is None and estimator is None:
            _raise(self.L.mcig_add_observable_default(self._h, int(kind), _dp(p), n, int(blocksize), int(nskip)))
            return
        if isinstance(estimator, bool):  # flag_correlated form (MCIntegrator.cpp:467-475)
            flag_error = blocksize > 0
            if estimator and not flag_error:
                raise ValueError("[selectEstimatorType] Error calculation is set off, but correlated error "
                                 "estimation is set on.")
            estimator = EST_CORRELATED if estimator else (EST_UNCORRELATED if flag_error else EST_NOOP)
        if estimator is None:
            estimator = EST_CORRELATED if blocksize == 1 else (EST_UNCORRELATED if blocksize > 0 else EST_NOOP)
        if flag_equil is None:
            flag_equil = blocksize > 0
        _raise(self.L.mcig_add_observable(self._h, int(kind), _dp(p), n, int(blocksize), int(nskip),
                                          int(bool(flag_equil)), int(estimator)))

    def popObservable(self):
        _raise(self.L.mcig_pop_observable(self._h))

    def clearObservables(self):
        _raise(self.L.mcig_clear_observables(self._h))

    def getNObs(self):
        n = ctypes.c_int()
        _raise(self.L.mcig_get_nobs(self._h, ctypes.byref(n)))
        return n.value

    def getNObsDim(self):
        n = ctypes.c_int()
        _raise(self.L.mcig_get_nobsdim(self._h, ctypes.byref(n)))
        return n.value

    def setFullStorage(self, bits):
        _raise(self.L.mcig_set_full_storage(self._h, int(bits)))

    # --- domain (MCIntegrator.hpp:129-137)
    def setIRange(self, lbounds, ubounds):
        lb = np.ascontiguousarray(np.broadcast_to(np.asarray(lbounds, dtype=np.float64), (self.ndim,)))
        ub = np.ascontiguousarray(np.broadcast_to(np.asarray(ubounds, dtype=np.float64), (self.ndim,)))
        _raise(self.L.mcig_set_irange(self._h, _dp(lb), _dp(ub)))

    def resetDomain(self):
        _raise(self.L.mcig_reset_domain(self._h))

    # --- integrate (MCIntegrator.hpp:225)
    def integrate(self, nmc, doFindMRT2step=True, doDecorrelation=True):
        nod = max(self.getNObsDim(), 1)
        avg = np.zeros(nod)
        err = np.zeros(nod)
        _raise(self.L.mcig_integrate(self._h, int(nmc), _dp(avg), _dp(err), int(bool(doFindMRT2step)),
                                     int(bool(doDecorrelation))))
        return avg[:self.getNObsDim()], err[:self.getNObsDim()]

    def integrate_into(self, nmc, avg, err, doFindMRT2step=True, doDecorrelation=True):
        """integrate() writing into caller-provided float64 arrays (no allocation per call)."""
        _raise(self.L.mcig_integrate(self._h, int(nmc), _dp(avg), _dp(err), int(bool(doFindMRT2step)),
                                     int(bool(doDecorrelation))))

    def getChainResults(self):
        nod = self.getNObsDim()
        a = np.zeros((self.nchains, max(nod, 1)))
        e = np.zeros((self.nchains, max(nod, 1)))
        _raise(self.L.mcig_get_chain_results(self._h, _dp(a), _dp(e)))
        return a[:, :nod], e[:, :nod]

    def getAcceptanceRate(self):
        v = ctypes.c_double()
        _raise(self.L.mcig_get_acceptance_rate(self._h, ctypes.byref(v)))
        return v.value

    def getCounts(self):
        a = np.zeros(self.nchains, dtype=np.int64)
        r = np.zeros(self.nchains, dtype=np.int64)
        _raise(self.L.mcig_get_counts(self._h, a.ctypes.data_as(P_int64), r.ctypes.data_as(P_int64)))
        return a, r

    def getObsData(self, o):
        """Accumulator data of observable o, [nchains][nstore*nobs] (AccumulatorInterface::getData)."""
        n = ctypes.c_int64()
        _raise(self.L.mcig_get_obs_data(self._h, int(o), None, ctypes.byref(n)))
        out = np.zeros(n.value)
        _raise(self.L.mcig_get_obs_data(self._h, int(o), _dp(out), ctypes.byref(n)))
        return out.reshape(self.nchains, -1)

    def getObsDataChains(self, o, c0, nc):
        """Accumulator data of observable o for the chains [c0, c0 + nc), [nc][nstore*nobs]."""
        n = ctypes.c_int64()
        _raise(self.L.mcig_get_obs_data_chains(self._h, int(o), int(c0), int(nc), None, ctypes.byref(n)))
        out = np.zeros(n.value)
        _raise(self.L.mcig_get_obs_data_chains(self._h, int(o), int(c0), int(nc), _dp(out), ctypes.byref(n)))
        return out.reshape(int(nc), -1)

    def getStepCounters(self):
        """Philox step counter of every chain (steps drawn since setSeed)."""
        out = np.zeros(self.nchains, dtype=np.uint64)
        _raise(self.L.mcig_get_step_counters(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
        return out

    def setReplay(self, tape, lens=None):
        if tape is None:
            _raise(self.L.mcig_set_replay(self._h, None, 0, None))
            self._tape = None
            return
        t = np.ascontiguousarray(np.asarray(tape, dtype=np.float64))
        if t.ndim == 1:
            t = t.reshape(1, -1)
        if lens is None:
            lens = np.full(t.shape[0], t.shape[1], dtype=np.int64)
        lens = np.ascontiguousarray(np.asarray(lens, dtype=np.int64))
        self._tape = (t, lens)
        _raise(self.L.mcig_set_replay(self._h, _dp(t), t.shape[1], lens.ctypes.data_as(P_int64)))

    def storeObservablesOnFile(self, path, freq):
        """MCI::storeObservablesOnFile: every freq-th main-sampling step of chain 0."""
        _raise(self.L.mcig_store_observables_on_file(self._h, str(path).encode(), int(freq)))

    def clearObservableFile(self):
        _raise(self.L.mcig_clear_observable_file(self._h))

    def storeWalkerPositionsOnFile(self, path, freq):
        """MCI::storeWalkerPositionsOnFile: every freq-th main-sampling step of chain 0."""
        _raise(self.L.mcig_store_walker_positions_on_file(self._h, str(path).encode(), int(freq)))

    def clearWalkerFile(self):
        _raise(self.L.mcig_clear_walker_file(self._h))

    def setRecordAccepts(self, on=True):
        _raise(self.L.mcig_set_record_accepts(self._h, int(bool(on))))

    def getAcceptBits(self):
        n = ctypes.c_int64()
        _raise(self.L.mcig_get_accept_bits(self._h, None, ctypes.byref(n)))
        out = np.zeros(n.value * self.nchains, dtype=np.uint8)
        _raise(self.L.mcig_get_accept_bits(self._h, out.ctypes.data_as(P_uint8), ctypes.byref(n)))
        return out.reshape(n.value, self.nchains)

    def getLastTimings(self):
        ms = np.zeros(4)
        n = ctypes.c_int64()
        _raise(self.L.mcig_get_last_timings(self._h, _dp(ms), ctypes.byref(n)))
        return {"calibration_ms": ms[0], "burnin_ms": ms[1], "sampling_ms": ms[2], "estimation_ms": ms[3],
                "launches": n.value}

    # --- snake_case aliases (shared test configuration, tests/golden/cases.py)
    def set_seeds(self, seeds):
        self.setSeed(int(np.asarray(seeds).ravel()[0]))

    set_irange = setIRange
    set_target_acceptance_rate = setTargetAcceptanceRate
    set_nfind_mrt2_iterations = setNfindMRT2Iterations
    set_ndecorrelation_steps = setNdecorrelationSteps
    set_multistep_move = setMultiStepMove
    multistep_add_pdf = addMultiStepSamplingFunction

    def add_sampling_function(self, kind, params=()):
        self.addSamplingFunction(kind, params)

    def set_trial_move(self, movetype, srrd=0, veclen=0, ntypes=1, type_ends=None):
        self.setTrialMove(movetype, srrd, veclen, ntypes, type_ends)

    def add_observable(self, kind, params=(), blocksize=1, nskip=1, flag_equil=None, estimator=None):
        self.addObservable(kind, params, blocksize, nskip, flag_equil, estimator)


class Flow:
    """Affine-coupling flow on the GPU (include/mcig.h, mcig_flow_*): the learned proposal."""

    def __init__(self, ndim, nlayers=8, hidden=128, seed=0, device=0):
        self.L = _lib.load()
        self.ndim = int(ndim)
        self.nlayers = int(nlayers)
        h = ctypes.c_void_p()
        _raise(self.L.mcig_flow_create(self.ndim, self.nlayers, int(hidden), ctypes.c_uint64(seed), int(device),
                                       ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.L.mcig_flow_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tensor_path(self, tc):
        """pass kernel: 0 (or False) register-fused mma.sync, 1 (or True) tcgen05 with TMEM
        accumulators, 2 mma.sync with the hidden activations in shared memory"""
        _raise(self.L.mcig_flow_set_tensor_path(self._h, int(tc)))

    def params(self):
        n = ctypes.c_int64()
        _raise(self.L.mcig_flow_get_params(self._h, None, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.float32)
        _raise(self.L.mcig_flow_get_params(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(n)))
        return out

    def set_params(self, theta):
        t = np.ascontiguousarray(np.asarray(theta, dtype=np.float32))
        _raise(self.L.mcig_flow_set_params(self._h, t.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), t.size))

    def _pass(self, fn, a):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
        out = np.zeros_like(a)
        lq = np.zeros(a.shape[0])
        _raise(fn(self._h, _dp(a), a.shape[0], _dp(out), _dp(lq)))
        return out, lq

    def forward(self, z):
        return self._pass(self.L.mcig_flow_forward, z)

    def inverse(self, x):
        return self._pass(self.L.mcig_flow_inverse, x)

    def loss_grad(self, x):
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
        g = np.zeros(self.L.mcig_flow_nparams(self.ndim, self.nlayers), dtype=np.float32)
        loss = ctypes.c_double()
        _raise(self.L.mcig_flow_loss_grad(self._h, _dp(x), x.shape[0], ctypes.byref(loss),
                                          g.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return loss.value, g

    def train(self, x, steps, batch, lr):
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
        loss = ctypes.c_double()
        _raise(self.L.mcig_flow_train(self._h, _dp(x), x.shape[0], int(steps), int(batch), float(lr), ctypes.byref(loss)))
        return loss.value


def integrate_flow(m, flow, nmc, period=5, refresh=0, train_steps=400, batch=2048, lr=2e-3, doFindMRT2step=True,
                   doDecorrelation=True):
    """MCI::integrate with the learned proposal (mcig_integrate_flow): `train_steps` adaptation
    cycles (period - 1 local steps + one Adam step on the current chain positions), then nmc
    recorded steps with a flow proposal every `period` steps.  Returns avg, err, flow acceptance."""
    nod = max(m.getNObsDim(), 1)
    avg = np.zeros(nod)
    err = np.zeros(nod)
    acc = ctypes.c_double()
    _raise(m.L.mcig_integrate_flow(m._h, flow._h, int(nmc), int(period), int(refresh), int(train_steps), int(batch),
                                   float(lr), _dp(avg), _dp(err), int(bool(doFindMRT2step)), int(bool(doDecorrelation)),
                                   ctypes.byref(acc)))
    return avg[:m.getNObsDim()], err[:m.getNObsDim()], acc.value


class Plugin:
    """User sampling functions and observables compiled for the device: a shared library
    built from a source that ends with MCIG_PLUGIN (include/mcig/plugin.cuh), e.g. with
    mcintegratorplusplus_gb300.build.build_plugin."""

    def __init__(self, path):
        self.L = _lib.load()
        h = ctypes.c_void_p()
        _raise(self.L.mcig_plugin_load(str(path).encode(), ctypes.byref(h)))
        self._h = h
        npdf, nobs = ctypes.c_int(), ctypes.c_int()
        _raise(self.L.mcig_plugin_counts(self._h, ctypes.byref(npdf), ctypes.byref(nobs)))
        self.npdf, self.nobs = npdf.value, nobs.value
        nmove = ctypes.c_int()
        _raise(self.L.mcig_plugin_nmoves(self._h, ctypes.byref(nmove)))
        self.nmove = nmove.value

    def pdf(self, k):
        """kind of the k-th sampling function"""
        return PDF_USER + int(k)

    def obs(self, k):
        """kind of the k-th observable"""
        return OBS_USER + int(k)


class Batch:
    """Many independent integrals (one MCI each) in one persistent launch (mcig_batch_*)."""

    def __init__(self, mcis, nmc, doFindMRT2step=True, doDecorrelation=True):
        self.L = _lib.load()
        self.mcis = list(mcis)
        arr = (ctypes.c_void_p * len(self.mcis))(*[m._h.value for m in self.mcis])
        nm = np.ascontiguousarray(np.broadcast_to(np.asarray(nmc, dtype=np.int64), (len(self.mcis),)))
        h = ctypes.c_void_p()
        _raise(self.L.mcig_batch_create(arr, len(self.mcis), nm.ctypes.data_as(P_int64), int(bool(doFindMRT2step)),
                                        int(bool(doDecorrelation)), ctypes.byref(h)))
        self._h = h
        self.nod = [m.getNObsDim() for m in self.mcis]

    def run(self):
        tot = sum(self.nod)
        avg = np.zeros(max(tot, 1))
        err = np.zeros(max(tot, 1))
        _raise(self.L.mcig_batch_run(self._h, _dp(avg), _dp(err)))
        out, off = [], 0
        for n in self.nod:
            out.append((avg[off:off + n].copy(), err[off:off + n].copy()))
            off += n
        return out

    def last_ms(self):
        v = ctypes.c_double()
        _raise(self.L.mcig_batch_last_ms(self._h, ctypes.byref(v)))
        return v.value

    def tuning(self):
        """(threads per block, [unroll of the four ndim buckets])"""
        blk = ctypes.c_int()
        u = (ctypes.c_int * 4)()
        _raise(self.L.mcig_batch_get_tuning(self._h, ctypes.byref(blk), u))
        return blk.value, list(u)

    def set_tuning(self, block, unroll=None):
        u = None if unroll is None else (ctypes.c_int * 4)(*[int(v) for v in unroll])
        _raise(self.L.mcig_batch_set_tuning(self._h, int(block), u))

    def autotune(self, cache_path=None):
        _raise(self.L.mcig_batch_autotune(self._h, cache_path.encode() if cache_path else None))
        return self.tuning()

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.L.mcig_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def estimate(estimator, x, device=0):
    """Reference estimator (src/Estimators.cpp) of x[n][ndim] computed on the GPU."""
    L = _lib.load()
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    n = x.shape[0]
    nd = 1 if x.ndim == 1 else x.shape[1]
    avg = np.zeros(nd)
    err = np.zeros(nd)
    _raise(L.mcig_estimate(int(device), int(estimator), n, nd, _dp(x), _dp(avg), _dp(err)))
    return avg, err


def accumulate_walk(obs_kind, xs, accepted, blocksize, nskip, params=(), device=0):
    """Accumulator of one observable driven by a recorded walk, on the GPU."""
    L = _lib.load()
    xs = np.ascontiguousarray(np.asarray(xs, dtype=np.float64))
    acc = np.ascontiguousarray(np.asarray(accepted, dtype=np.uint8))
    p, npar = _params(params)
    n = ctypes.c_int64()
    nsteps, nd = xs.shape
    _raise(L.mcig_accumulate_walk(int(device), int(obs_kind), _dp(p), npar, nd, int(blocksize), int(nskip), nsteps,
                                  _dp(xs), acc.ctypes.data_as(P_uint8), None, ctypes.byref(n)))
    out = np.zeros(n.value)
    _raise(L.mcig_accumulate_walk(int(device), int(obs_kind), _dp(p), npar, nd, int(blocksize), int(nskip), nsteps,
                                  _dp(xs), acc.ctypes.data_as(P_uint8), _dp(out), ctypes.byref(n)))
    return out


def philox_block(ctr, key, device=0):
    L = _lib.load()
    c = (ctypes.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in ctr])
    k = (ctypes.c_uint32 * 2)(*[int(v) & 0xFFFFFFFF for v in key])
    o = (ctypes.c_uint32 * 4)()
    _raise(L.mcig_philox_block(int(device), c, k, o))
    return [o[i] for i in range(4)]
