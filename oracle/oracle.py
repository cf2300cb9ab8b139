"""ctypes binding of the CPU oracle (oracle/mci_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py.  The product package never imports this module.

`OracleMCI` mirrors the reference's ``mci::MCI`` interface
(include/mci/MCIntegrator.hpp:93-225) with one reference MCI object per chain.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")

_c_int64_p = ctypes.POINTER(ctypes.c_int64)
_c_double_p = ctypes.POINTER(ctypes.c_double)


def build(force=False):
    """Compile oracle/mci_oracle.c into oracle/_build/liboracle.so (gcc, no FMA contraction)."""
    src = os.path.join(HERE, "mci_oracle.c")
    hdr = os.path.join(HERE, "mci_oracle.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) > max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
                           src, "-o", tmp, "-lm", "-lpthread"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int, ctypes.c_int]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_get_acceptance_rate.restype = ctypes.c_double
        L.orc_get_acceptance_rate.argtypes = [ctypes.c_void_p]
        for name in ("orc_get_tape", "orc_get_accept_bits", "orc_get_obs_data", "orc_accumulate_walk",
                     "orc_get_margins"):
            getattr(L, name).restype = ctypes.c_int64
        L.orc_set_ndecorrelation_steps.argtypes = [ctypes.c_void_p, ctypes.c_int64]
        L.orc_set_philox.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int]
        L.orc_get_margins.argtypes = [ctypes.c_void_p, ctypes.c_int, _c_double_p, ctypes.c_int64]
        L.orc_set_mrt2step.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.orc_set_mrt2step_i.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
        L.orc_set_target_acceptance_rate.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.orc_set_multistep_move.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_double]
        L.orc_integrate.argtypes = [ctypes.c_void_p, ctypes.c_int64, _c_double_p, _c_double_p, ctypes.c_int,
                                    ctypes.c_int, _c_double_p, _c_double_p, ctypes.c_int]
        _LIB = L
    return _LIB


def _dp(a):
    return a.ctypes.data_as(_c_double_p)


class OracleError(RuntimeError):
    pass


def _check(rc):
    if rc != 0:
        raise OracleError("oracle error %d: %s" % (rc, lib().orc_last_error().decode()))


class OracleMCI:
    """One reference MCI per chain; seeds are given per chain."""

    def __init__(self, ndim, nchains=1):
        self.L = lib()
        self.ndim = ndim
        self.nchains = nchains
        self.h = self.L.orc_create(ndim, nchains)
        if not self.h:
            raise OracleError(self.L.orc_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(ctypes.c_void_p(self.h))
            self.h = None

    def _hv(self):
        return ctypes.c_void_p(self.h)

    def set_seeds(self, seeds):
        s = np.ascontiguousarray(np.broadcast_to(np.asarray(seeds, dtype=np.uint64), (self.nchains,)))
        _check(self.L.orc_set_seeds(self._hv(), s.ctypes.data_as(ctypes.c_void_p)))

    def set_x(self, x):
        x = np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), (self.nchains, self.ndim)))
        _check(self.L.orc_set_x(self._hv(), _dp(x)))

    def get_x(self):
        x = np.zeros((self.nchains, self.ndim))
        _check(self.L.orc_get_x(self._hv(), _dp(x)))
        return x

    def set_mrt2step(self, v, i=None):
        if i is None:
            _check(self.L.orc_set_mrt2step(self._hv(), float(v)))
        else:
            _check(self.L.orc_set_mrt2step_i(self._hv(), int(i), float(v)))

    def get_mrt2step(self, chain=0, i=0):
        v = ctypes.c_double()
        _check(self.L.orc_get_mrt2step(self._hv(), chain, i, ctypes.byref(v)))
        return v.value

    def set_target_acceptance_rate(self, r):
        _check(self.L.orc_set_target_acceptance_rate(self._hv(), float(r)))

    def set_nfind_mrt2_iterations(self, n):
        _check(self.L.orc_set_nfind_mrt2_iterations(self._hv(), int(n)))

    def set_ndecorrelation_steps(self, n):
        _check(self.L.orc_set_ndecorrelation_steps(self._hv(), int(n)))

    def set_trial_move(self, movetype, srrd=0, veclen=0, ntypes=1, type_ends=None):
        te = None if type_ends is None else (ctypes.c_int * len(type_ends))(*type_ends)
        _check(self.L.orc_set_trial_move(self._hv(), movetype, srrd, veclen, ntypes, te))

    def set_multistep_move(self, nsteps, sub_srrd=0, sub_veclen=1, sub_step=0.05):
        _check(self.L.orc_set_multistep_move(self._hv(), nsteps, sub_srrd, sub_veclen, float(sub_step)))

    def multistep_add_pdf(self, kind, params=()):
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float64).ravel())
        _check(self.L.orc_multistep_add_pdf(self._hv(), kind, _dp(p), p.size))

    def add_sampling_function(self, kind, params=()):
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float64).ravel())
        _check(self.L.orc_add_sampling_function(self._hv(), kind, _dp(p), p.size))

    def add_observable(self, kind, params=(), blocksize=1, nskip=1, flag_equil=None, estimator=None):
        if flag_equil is None:
            flag_equil = blocksize > 0
        if estimator is None:  # addObservable(obs, blocksize, nskip) defaults (MCIntegrator.hpp:161-164)
            estimator = 2 if blocksize == 1 else (1 if blocksize > 0 else 0)
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float64).ravel())
        _check(self.L.orc_add_observable(self._hv(), kind, _dp(p), p.size, blocksize, nskip,
                                         int(bool(flag_equil)), estimator))

    def clear_observables(self):
        _check(self.L.orc_clear_observables(self._hv()))

    def nobsdim(self):
        return self.L.orc_get_nobsdim(self._hv())

    def set_irange(self, lb, ub):
        lb = np.ascontiguousarray(np.broadcast_to(np.asarray(lb, dtype=np.float64), (self.ndim,)))
        ub = np.ascontiguousarray(np.broadcast_to(np.asarray(ub, dtype=np.float64), (self.ndim,)))
        _check(self.L.orc_set_irange(self._hv(), _dp(lb), _dp(ub)))

    def set_record(self, on=True):
        _check(self.L.orc_set_record(self._hv(), int(on)))

    def get_tape(self, chain=0):
        n = self.L.orc_get_tape(self._hv(), chain, None, 0)
        out = np.zeros(n)
        self.L.orc_get_tape(self._hv(), chain, _dp(out), n)
        return out

    def get_tapes(self):
        """All chains' tapes as one [nchains][stride] array plus per-chain lengths."""
        tapes = [self.get_tape(c) for c in range(self.nchains)]
        lens = np.array([len(t) for t in tapes], dtype=np.int64)
        stride = int(lens.max()) if len(lens) else 0
        out = np.zeros((self.nchains, max(stride, 1)))
        for c, t in enumerate(tapes):
            out[c, :len(t)] = t
        return out, lens

    def get_accept_bits(self, chain=0):
        ms = ctypes.c_int64()
        n = self.L.orc_get_accept_bits(self._hv(), chain, None, 0, ctypes.byref(ms))
        out = np.zeros(n, dtype=np.uint8)
        self.L.orc_get_accept_bits(self._hv(), chain, out.ctypes.data_as(ctypes.c_void_p), n, ctypes.byref(ms))
        return out, ms.value

    def set_replay(self, tape, lens):
        self._tape = np.ascontiguousarray(tape, dtype=np.float64)
        self._lens = np.ascontiguousarray(lens, dtype=np.int64)
        _check(self.L.orc_set_replay(self._hv(), _dp(self._tape), self._tape.shape[1],
                                     self._lens.ctypes.data_as(_c_int64_p)))

    def set_philox(self, seed, chain0=0, ctr0=None, layout=1):
        """Draw from the device kernels' Philox streams (layout 1: float kernels, 2: double
        kernels, 0: back to std::mt19937_64): chain c is device chain chain0 + c."""
        self._ctr0 = None if ctr0 is None else np.ascontiguousarray(np.asarray(ctr0, dtype=np.uint64))
        _check(self.L.orc_set_philox(self._hv(), ctypes.c_uint64(int(seed)), ctypes.c_int64(int(chain0)),
                                     None if self._ctr0 is None else self._ctr0.ctypes.data_as(ctypes.c_void_p),
                                     int(layout)))

    def philox_counters(self):
        out = np.zeros(self.nchains, dtype=np.uint64)
        _check(self.L.orc_get_philox_counters(self._hv(), out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def set_chain_steps(self, steps):
        """Per-chain step sizes, [nchains][ntypes]."""
        st = np.ascontiguousarray(np.asarray(steps, dtype=np.float64).reshape(self.nchains, -1))
        _check(self.L.orc_set_chain_steps(self._hv(), _dp(st)))

    def get_margins(self, chain=0):
        """log(u) - log(acceptance) of every recorded step (accepted iff <= 0), aligned with get_accept_bits."""
        n = self.L.orc_get_margins(self._hv(), chain, None, 0)
        out = np.zeros(n)
        self.L.orc_get_margins(self._hv(), chain, _dp(out), n)
        return out

    def integrate(self, nmc, do_find=True, do_decorr=True, nthreads=1, per_chain=False):
        nod = max(self.nobsdim(), 1)
        avg = np.zeros(nod)
        err = np.zeros(nod)
        ca = np.zeros((self.nchains, nod)) if per_chain else None
        ce = np.zeros((self.nchains, nod)) if per_chain else None
        _check(self.L.orc_integrate(self._hv(), int(nmc), _dp(avg), _dp(err), int(do_find), int(do_decorr),
                                    _dp(ca) if per_chain else None, _dp(ce) if per_chain else None, nthreads))
        if per_chain:
            return avg, err, ca, ce
        return avg, err

    def acceptance_rate(self):
        return self.L.orc_get_acceptance_rate(self._hv())

    def counts(self):
        a = np.zeros(self.nchains, dtype=np.int64)
        r = np.zeros(self.nchains, dtype=np.int64)
        _check(self.L.orc_get_counts(self._hv(), a.ctypes.data_as(_c_int64_p), r.ctypes.data_as(_c_int64_p)))
        return a, r

    def obs_data(self, o):
        n = self.L.orc_get_obs_data(self._hv(), o, None, 0)
        out = np.zeros(max(n, 0))
        self.L.orc_get_obs_data(self._hv(), o, _dp(out), n)
        return out.reshape(self.nchains, -1)


def estimate(estimator, x):
    """Reference estimator on x[n][ndim] (or x[n])."""
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    n = x.shape[0]
    nd = 1 if x.ndim == 1 else x.shape[1]
    avg = np.zeros(nd)
    err = np.zeros(nd)
    _check(lib().orc_estimate(estimator, ctypes.c_int64(n), nd, _dp(x), _dp(avg), _dp(err)))
    return avg, err


def block_estimate(x, nblocks):
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    n = x.shape[0]
    nd = 1 if x.ndim == 1 else x.shape[1]
    avg = np.zeros(nd)
    err = np.zeros(nd)
    _check(lib().orc_block_estimate(ctypes.c_int64(n), nd, _dp(x), ctypes.c_int64(nblocks), _dp(avg), _dp(err)))
    return avg, err


def accumulate_walk(obs_kind, xs, accepted, blocksize, nskip, params=()):
    xs = np.ascontiguousarray(np.asarray(xs, dtype=np.float64))
    acc = np.ascontiguousarray(np.asarray(accepted, dtype=np.uint8))
    p = np.ascontiguousarray(np.asarray(params, dtype=np.float64).ravel())
    n, nd = xs.shape
    out = np.zeros(n * max(nd, 8) + 16)
    m = lib().orc_accumulate_walk(obs_kind, _dp(p), p.size, nd, blocksize, nskip, ctypes.c_int64(n), _dp(xs),
                                  acc.ctypes.data_as(ctypes.c_void_p), _dp(out), ctypes.c_int64(out.size))
    if m < 0:
        raise OracleError(lib().orc_last_error().decode())
    return out[:m]


def mt64_stream(seed, n):
    out = np.zeros(n, dtype=np.uint64)
    lib().orc_mt64_stream(ctypes.c_uint64(seed), ctypes.c_int64(n), out.ctypes.data_as(ctypes.c_void_p))
    return out


def canonical_stream(seed, n):
    out = np.zeros(n)
    lib().orc_canonical_stream(ctypes.c_uint64(seed), ctypes.c_int64(n), _dp(out))
    return out


def normal_stream(seed, n):
    out = np.zeros(n)
    lib().orc_normal_stream(ctypes.c_uint64(seed), ctypes.c_int64(n), _dp(out))
    return out


def uniform_int_stream(seed, n, nvals):
    out = np.zeros(n, dtype=np.int64)
    lib().orc_uniform_int_stream(ctypes.c_uint64(seed), ctypes.c_int64(n), ctypes.c_int64(nvals),
                                 out.ctypes.data_as(_c_int64_p))
    return out


def srrd_stream(srrd, seed, n):
    """n draws of SRRDType srrd (createSymRRD's default distribution) from a fresh object."""
    out = np.zeros(n)
    lib().orc_srrd_stream(int(srrd), ctypes.c_uint64(seed), ctypes.c_int64(n), _dp(out))
    return out


def philox4x32_10(ctr, key):
    c = (ctypes.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in ctr])
    k = (ctypes.c_uint32 * 2)(*[int(v) & 0xFFFFFFFF for v in key])
    o = (ctypes.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return [o[i] for i in range(4)]


def splitmix64_ar1(seed, n, nd, phi):
    """The deterministic AR(1) test series of oracle/ref_recorder.cpp (ar1_series)."""
    mask = (1 << 64) - 1
    s = seed
    x = np.zeros((n, nd))
    for i in range(n):
        for j in range(nd):
            s = (s + 0x9E3779B97F4A7C15) & mask
            z = s
            z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
            z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
            z = z ^ (z >> 31)
            u = float(z >> 11) * (1.0 / 9007199254740992.0)
            prev = x[i - 1, j] if i > 0 else 0.0
            x[i, j] = phi * prev + (u - 0.5)
    return x


def splitmix64_walk(seed, accept_seed, n, nd, phi):
    """Walk of oracle/ref_recorder.cpp: AR(1) positions, about 1/3 of steps rejected (position repeated)."""
    mask = (1 << 64) - 1
    x = splitmix64_ar1(seed, n, nd, phi)
    acc = np.zeros(n, dtype=np.uint8)
    s = accept_seed
    acc[0] = 1
    for i in range(1, n):
        s = (s + 0x9E3779B97F4A7C15) & mask
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        z = z ^ (z >> 31)
        a = z % 3 != 0
        acc[i] = 1 if a else 0
        if not a:
            x[i] = x[i - 1]
    return x, acc
