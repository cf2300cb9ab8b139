"""Integration cases recorded from the reference by oracle/ref_recorder.cpp.

Each entry restates one RunSpec of the recorder so that any backend with the
MCI-style interface (the oracle's OracleMCI or the device mcintegratorplusplus_gb300.MCI)
can be configured identically.  The configuration order follows the recorder:
seed, domain, sampling function, trial move, target rate, calibration and
burn-in settings, observables; then integrate(0, find, decorr) followed by
integrate(nmc, no find, no decorr).
"""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN_PATH = os.path.join(HERE, "reference_golden.json")

# enum values of include/mcig_types.h
PDF_GAUSS_SUM, PDF_GAUSS, PDF_EXP = 0, 1, 2
OBS_X2SUM, OBS_XND, OBS_X2, OBS_X2MEAN, OBS_CONST, OBS_POLYNOM, OBS_X2BLOCK, OBS_GAUSSX2, OBS_XI, OBS_LOGPDF = range(10)
MOVE_ALL, MOVE_VEC, MOVE_MULTISTEP = 0, 1, 2
SRRD_UNIFORM, SRRD_GAUSSIAN = 0, 1
EST_NOOP, EST_UNCORRELATED, EST_CORRELATED, EST_FCBLOCKER, EST_MJBLOCKER = range(5)

# name, ndim, seed, move, veclen, pdf, obsset, blocksize, nskip, estim, nfind, ndecorr, nmc, periodic, target, nbits
RUNS = [
    ("c1_seed1234", 3, 1234, 0, 0, 0, 0, 1024, 1, EST_MJBLOCKER, -50, 1000, 1 << 20, 0, 0.5, 16384),
    ("all_uniform_full", 3, 5649871, 0, 0, 1, 1, 1, 1, -1, 20, 2000, 16384, 0, 0.5, 16384),
    ("all_gauss_block", 3, 1337, 1, 0, 0, 0, 16, 1, -1, 20, 2000, 16384, 0, 0.5, 16384),
    ("vec1_uniform", 3, 1337, 2, 1, 0, 2, 1, 3, -1, -50, 1000, 3 * 8192, 0, 0.5, 16384),
    ("vec3_gauss_nd6", 6, 77, 5, 3, 0, 0, 1, 2, -1, -50, 500, 8192, 0, 0.5, 8192),
    ("typed_all", 3, 1337, 4, 0, 0, 2, 8, 2, -1, -50, 1000, 16384, 0, 0.5, 16384),
    ("multistep_exp", 3, 1337, 3, 0, 0, 2, 1, 1, -1, -50, 500, 8192, 0, 0.85, 8192),
    ("exp_pdf_simple", 4, 31337, 0, 0, 2, 0, 0, 1, -1, -50, 500, 8192, 0, 0.5, 8192),
    ("periodic_3dgauss", 3, 5649871, 0, 0, 1, 1, 1, 1, -1, 10, 1000, 10000, 1, 0.5, 4096),
    ("nopdf_periodic", 3, 5649871, 0, 0, 3, 3, 1, 1, EST_UNCORRELATED, 0, 0, 10000, 1, 0.5, 64),
    ("auto_decorr", 3, 2024, 0, 0, 0, 0, 1, 1, -1, -50, -10000, 8192, 0, 0.5, 8192),
    # move 10 + k: SRRDType k (all coordinates, or single-coordinate vector moves with veclen 1)
    ("srrd_student_all", 3, 211, 12, 0, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096),
    ("srrd_cauchy_all", 3, 311, 13, 0, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096),
    ("srrd_exponential_vec1", 4, 411, 14, 1, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096),
    ("srrd_gamma_all", 3, 511, 15, 0, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096),
    ("srrd_weibull_all", 3, 611, 16, 0, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096),
    ("srrd_lognormal_all", 3, 711, 17, 0, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096),
    ("srrd_chisq_vec1", 4, 811, 18, 1, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096),
    ("srrd_fisher_all", 3, 911, 19, 0, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096),
]

FIELDS = ("name", "ndim", "seed", "move", "veclen", "pdf", "obsset", "blocksize", "nskip", "estim",
          "nfind", "ndecorr", "nmc", "periodic", "target", "nbits")


def runs():
    return [dict(zip(FIELDS, r)) for r in RUNS]


def run(name):
    for r in runs():
        if r["name"] == name:
            return r
    raise KeyError(name)


def golden():
    with open(GOLDEN_PATH) as f:
        return json.load(f)


def unpack_bits(hexstr, n):
    """Inverse of bits_hex in oracle/ref_recorder.cpp (4 bits per hex digit, LSB first)."""
    out = []
    for ch in hexstr:
        v = int(ch, 16)
        for j in range(4):
            out.append((v >> j) & 1)
    return out[:n]


def configure(m, r, set_seed):
    """Configure an MCI-style object m as the recorder configures the reference for run r.

    set_seed(m, seed) seeds the object (oracle: one mt19937_64 seed per chain)."""
    nd = r["ndim"]
    set_seed(m, r["seed"])
    if r["periodic"]:
        m.set_irange([-2.5] * nd, [2.5] * nd)
    pdf = r["pdf"]
    if pdf == 0:
        m.add_sampling_function(PDF_GAUSS)
    elif pdf == 1:
        m.add_sampling_function(PDF_GAUSS_SUM)
    elif pdf == 2:
        m.add_sampling_function(PDF_EXP)
    mv = r["move"]
    if mv == 1:
        m.set_trial_move(MOVE_ALL, SRRD_GAUSSIAN, 0)
    elif mv == 2:
        m.set_trial_move(MOVE_VEC, SRRD_UNIFORM, r["veclen"])
    elif mv == 3:
        m.set_multistep_move(nd, SRRD_UNIFORM, 1, 0.1)
        m.multistep_add_pdf(PDF_EXP)
    elif mv == 4:
        m.set_trial_move(MOVE_ALL, SRRD_UNIFORM, 0, 2, [1, nd])
    elif mv == 5:
        m.set_trial_move(MOVE_VEC, SRRD_GAUSSIAN, r["veclen"])
    elif mv >= 10:
        m.set_trial_move(MOVE_VEC if r["veclen"] else MOVE_ALL, mv - 10, r["veclen"])
    m.set_target_acceptance_rate(r["target"])
    m.set_nfind_mrt2_iterations(r["nfind"])
    m.set_ndecorrelation_steps(r["ndecorr"])
    obs = {0: [OBS_X2SUM, OBS_XND], 1: [OBS_X2MEAN], 2: [OBS_X2SUM, OBS_X2], 3: [OBS_GAUSSX2]}[r["obsset"]]
    for k in obs:
        if r["estim"] < 0:
            m.add_observable(k, (), r["blocksize"], r["nskip"])
        else:
            m.add_observable(k, (), r["blocksize"], r["nskip"], False, r["estim"])
