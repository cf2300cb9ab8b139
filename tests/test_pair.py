"""Two-lane kernel (mcig_pair.cuh): one exp(-x.x) or precision-matrix sampling function in
9..16 coordinates with two lanes per chain.

Bit-identity: the kernel gives the one-lane register-resident kernel's results bit for bit
(step sizes, walkers, Philox counters, acceptance counts, every accumulator value, averages
and errors), for Kahan-float and double sums, uniform and Gaussian moves, a partial last
warp (chain counts that are not a multiple of 16) and zero-padded coordinates (ndim < 16):
the lanes only share a chain's step.  The one-lane kernel is itself held to the FP64 oracle
on the same Philox draws (tests/test_fast_vs_oracle.py), so the same holds for this one.
Also the analytic check of the benchmark workload through it: x.x within 3 standard errors
(from the spread of the chain means) of tr Sigma, every coordinate mean within 3 of 0.
Reference: MCI::doStepMRT2 / sample (src/MCIntegrator.cpp:290-360).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def target(ndim, seed=2024):
    rng = np.random.default_rng(seed)
    Q, R = np.linalg.qr(rng.standard_normal((ndim, ndim)))
    Q = Q * np.sign(np.diag(R))
    lam = 10.0 ** rng.uniform(-1.0, 1.0, ndim)
    Sigma = Q @ np.diag(lam) @ Q.T
    P = Q @ np.diag(1.0 / lam) @ Q.T
    return Sigma, 0.5 * (P + P.T)


def configure(m, ndim, pdf, srrd, nmc, nblocks, obsset="all"):
    if pdf == "prec":
        m.add_sampling_function(3, target(ndim)[1])   # GAUSS_PREC
    else:
        m.add_sampling_function(1, ())                # exp(-x.x)
    m.set_trial_move(0, srrd, 0)                      # all-coordinate move
    m.set_nfind_mrt2_iterations(-50)
    m.set_ndecorrelation_steps(300)
    bs = nmc // nblocks
    m.add_observable(0, (), bs, 1, False, 1)   # x.x Block
    m.add_observable(1, (), bs, 1, False, 1)   # x_i Block
    m.add_observable(0, (), 1, 1, False, 1)    # x.x Full
    if obsset == "moments":                    # x and x.x only: the kernels' variants for them
        m.add_observable(1, (), 1, 1, False, 1)
        return
    if pdf == "prec":
        m.add_observable(1, (), 1, 1, False, 1)    # x_i Full
    else:
        m.add_observable(2, (), 1, 2, False, 1)    # x_i^2 Full, every 2nd step
    m.add_observable(8, (ndim - 1,), 0, 1, False, 0)  # x_(ndim-1) Simple
    m.add_observable(9, (), 0, 1, False, 0)    # log p Simple
    m.add_observable(5, (), bs, 1, False, 1)   # sum x_i Block


def run(mcig, prec, lanes, ndim, pdf, srrd, nc, nmc=1200, nblocks=12, seed=77, split=True, obsset="all"):
    m = mcig.MCI(ndim, nc, device=0, precision=prec)
    m.setSeed(seed)
    m.setFullStorage(32)
    configure(m, ndim, pdf, srrd, nmc, nblocks, obsset)
    m.setCalibrationSplit(split)
    if lanes:
        m.setLanes(lanes)
    else:
        m.setKernel(2)
    avg, err = m.integrate(nmc)
    ca, ce = m.getChainResults()
    out = {"avg": avg, "err": err, "ca": ca, "ce": ce, "steps": m.getMRT2Steps(), "x": m.getX(),
           "ctr": m.getStepCounters(), "counts": np.stack(m.getCounts())}
    for o in range(m.getNObs()):
        out["data%d" % o] = m.getObsData(o)
    return out


@pytest.mark.parametrize("prec_name,ndim,pdf,srrd,nc,split,obsset", [
    ("fp32", 16, "prec", 1, 1000, True, "all"),         # partial last warp, every served observable kind
    ("fp32_acc64", 16, "prec", 1, 1000, True, "all"),   # double block sums
    ("fp32", 11, "prec", 0, 520, True, "all"),          # padded coordinates, uniform move
    ("fp32", 13, "gauss", 1, 777, True, "all"),         # exp(-x.x)
    ("fp32", 16, "prec", 1, 600, False, "all"),         # calibration on two lanes as well
    ("fp32", 16, "prec", 1, 1000, True, "moments"),     # the benchmark's observables (x, x.x variants)
    ("fp32_acc64", 13, "gauss", 1, 520, True, "moments"),
])
def test_pair_bit_identical_to_one_lane(prec_name, ndim, pdf, srrd, nc, split, obsset):
    import mcintegratorplusplus_gb300 as mcig
    prec = {"fp32": mcig.PREC_FP32, "fp32_acc64": mcig.PREC_FP32_ACC64}[prec_name]
    a = run(mcig, prec, 0, ndim, pdf, srrd, nc, split=split, obsset=obsset)
    b = run(mcig, prec, 2, ndim, pdf, srrd, nc, split=split, obsset=obsset)
    for k in a:
        assert np.array_equal(a[k], b[k]), (k, np.max(np.abs(np.asarray(a[k], float) - np.asarray(b[k], float))))


def test_pair_analytic_benchmark_form():
    """65,536-chain benchmark form on 4,096 chains: x.x against tr Sigma, x_i against 0."""
    import mcintegratorplusplus_gb300 as mcig
    ndim, nc, nmc = 16, 4096, 4000
    Sigma, P = target(ndim)
    m = mcig.MCI(ndim, nc, device=0, precision=mcig.PREC_FP32)
    m.setSeed(20241203)
    m.setFullStorage(32)
    m.add_sampling_function(3, P)
    m.set_trial_move(0, 1, 0)
    m.set_nfind_mrt2_iterations(-50)
    m.set_ndecorrelation_steps(1000)
    m.add_observable(0, (), nmc // 40, 1, False, 1)
    m.add_observable(1, (), nmc // 40, 1, False, 1)
    m.setLanes(2)
    m.integrate(nmc)
    ca, _ = m.getChainResults()
    tr = float(np.trace(Sigma))
    z_xx = (ca[:, 0].mean() - tr) / (ca[:, 0].std(ddof=1) / np.sqrt(nc))
    assert abs(z_xx) < 3.0, z_xx
    zi = ca[:, 1:].mean(0) / (ca[:, 1:].std(0, ddof=1) / np.sqrt(nc))
    assert np.all(np.abs(zi) < 3.5), zi
