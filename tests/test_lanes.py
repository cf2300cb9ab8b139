"""Multi-lane mixture kernel (mcig_lanes.cuh) and the FP64-certified Metropolis decision.

* Bit-identity: the kernel with 4 or 8 lanes per chain gives the one-lane kernel's results
  bit for bit (step sizes, walkers, Philox counters, every accumulator value, averages and
  errors), for Kahan-float and double sums: the lanes only share a chain's work.
* FP64 decision: with the double test on every step (mode 2), every float decision that the
  double test reverses has a float margin below the certification band's lower edge
  2^-12, so mode 1 (double only inside the band) takes the same decisions as mode 2.
* Against the FP64 oracle on the same Philox draws (the precision form's "error against an
  FP64 oracle"): from the device's burnt-in state, the oracle (double walker, reference
  formula) follows the float walker step for step until a near-tie.
* Against the analytic moments of the mixture (x.x, x_i, x_i^2) within 3 standard errors
  from the spread of the chain means.
"""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu

NDIM, NCOMP = 32, 8


def mixture(seed=404):
    rng = np.random.default_rng(seed)
    means = rng.standard_normal((NCOMP, NDIM)) * 3.0
    widths = 10.0 ** rng.uniform(np.log10(0.3), np.log10(3.0), (NCOMP, NDIM))
    w = rng.dirichlet(np.ones(NCOMP))
    params = np.concatenate([[NCOMP], w, means.ravel(), widths.ravel()])
    m1 = (w[:, None] * means).sum(0)
    m2 = (w[:, None] * (widths ** 2 + means ** 2)).sum(0)
    return params, w, means, widths, m1, m2


def start(nc, seed=1):
    _, w, means, widths, _, _ = mixture()
    rng = np.random.default_rng(seed)
    comp = rng.choice(NCOMP, nc, p=w)
    return means[comp] + widths[comp] * rng.standard_normal((nc, NDIM))


def configure(m, nmc, nblocks=16, moments=False):
    """The mixture configuration; moments: x.x, x_i, x_i^2 in Block accumulators only, else
    a mix of every observable kind and accumulator the multi-lane kernel serves (at most
    2 ndim + 8 observable values)."""
    params = mixture()[0]
    m.add_sampling_function(5, params)        # GAUSS_MIX
    m.set_trial_move(0, 1, 0)                 # all-coordinate, Gaussian
    m.set_nfind_mrt2_iterations(-50)
    m.set_ndecorrelation_steps(256)
    bs = nmc // nblocks
    m.add_observable(0, (), bs, 1, False, 1)  # x.x Block
    m.add_observable(1, (), bs, 1, False, 1)  # x_i Block
    if moments:
        m.add_observable(2, (), bs, 1, False, 1)  # x_i^2 Block
        return
    m.add_observable(1, (), 1, 1, False, 1)   # x_i Full
    m.add_observable(8, (5,), 1, 2, False, 1)  # x_5 Full, every 2nd step
    m.add_observable(9, (), 0, 1, False, 0)   # log p Simple
    m.add_observable(5, (), 0, 1, False, 0)   # sum x_i Simple
    m.add_observable(3, (), 1, 1, False, 1)   # x.x / ndim Full


def run(mcig, prec, lanes, nc=512, nmc=2048, f64=0, seed=31, moments=False):
    m = mcig.MCI(NDIM, nc, device=0, precision=prec)
    m.setSeed(seed)
    m.setFullStorage(32)
    configure(m, nmc, moments=moments)
    m.setX(start(nc))
    if lanes:
        m.setLanes(lanes)
        m.setKernel(3)
    else:
        m.setKernel(2)
    if f64:
        m.setFP64Decision(f64)
    avg, err = m.integrate(nmc)
    ca, ce = m.getChainResults()
    out = {"avg": avg, "err": err, "ca": ca, "ce": ce, "steps": m.getMRT2Steps(), "x": m.getX(),
           "ctr": m.getStepCounters(), "counts": np.stack(m.getCounts())}
    for o in range(m.getNObs()):
        out["data%d" % o] = m.getObsData(o)
    out["stats"] = m.getDecisionStats() if f64 else None
    return out


@pytest.mark.parametrize("prec_name", ["fp32", "fp32_acc64"])
@pytest.mark.parametrize("lanes", [4, 8])
def test_lanes_bit_identical_to_one_lane(prec_name, lanes):
    import mcintegratorplusplus_gb300 as mcig
    prec = {"fp32": mcig.PREC_FP32, "fp32_acc64": mcig.PREC_FP32_ACC64}[prec_name]
    a = run(mcig, prec, 0)
    b = run(mcig, prec, lanes)
    for k in a:
        if a[k] is None:
            continue
        assert np.array_equal(a[k], b[k]), (k, np.max(np.abs(np.asarray(a[k], float) - np.asarray(b[k], float))))


def test_fp64_decision_band():
    import mcintegratorplusplus_gb300 as mcig
    every = run(mcig, mcig.PREC_FP32, 8, f64=2)
    band = run(mcig, mcig.PREC_FP32, 8, f64=1)
    plain = run(mcig, mcig.PREC_FP32, 8, f64=0)
    checked, reversed_, margin = every["stats"]
    steps = int(every["ctr"].sum())  # every step of every chain (calibration, burn-in, sampling)
    assert checked == steps, (checked, steps)
    assert margin < 2.0 ** -12, margin  # reversals lie inside the band of mode 1
    nb, rb, mb = band["stats"]
    assert 0 < nb < 0.01 * steps, (nb, steps)  # mode 1 tests few steps in double
    for k in every:
        if k != "stats":
            assert np.array_equal(every[k], band[k]), k
    if reversed_ == 0:  # no float decision differs: the float run is the same walk
        assert np.array_equal(plain["x"], band["x"])
    print("\nFP64 decision: %d steps, %d tested in double in the band (%.2e), %d float decisions reversed, "
          "largest reversed float margin %.3e" % (steps, nb, nb / steps, reversed_, margin))


def test_lanes_fp64_decision_against_fp64_oracle_same_draws():
    import mcintegratorplusplus_gb300 as mcig
    nc, nmc, K = 256, 4096, 32
    m = mcig.MCI(NDIM, nc, device=0, precision=mcig.PREC_FP32)
    m.setSeed(77)
    m.setFullStorage(32)
    configure(m, nmc)
    m.setX(start(nc, seed=3))
    m.setLanes(8)
    m.setKernel(3)
    m.setFP64Decision(1)
    m.integrate(0, True, True)  # calibration and burn-in
    x, steps, ctr = m.getX(), m.getMRT2Steps(), m.getStepCounters()
    m.integrate(nmc, False, False)
    ca, _ = m.getChainResults()
    o = orc.OracleMCI(NDIM, K)
    configure(o, nmc)
    o.set_x(x[:K])
    o.set_chain_steps(steps[:K])
    o.set_philox(77, 0, ctr[:K], layout=1)
    o.set_record(True)
    _, _, oca, _ = o.integrate(nmc, False, False, nthreads=8, per_chain=True)
    xs_dev = m.getObsDataChains(2, 0, K).reshape(K, nmc, NDIM)  # x_i Full
    xs_orc = o.obs_data(2).reshape(K, nmc, NDIM)
    first = np.full(K, nmc)
    for c in range(K):
        bits, s0 = o.get_accept_bits(c)
        mg = o.get_margins(c)[s0:s0 + nmc]
        d = np.max(np.abs(xs_dev[c] - xs_orc[c]), axis=1)
        apart = np.nonzero(d > 1e-2)[0]
        if apart.size:
            t = int(apart[0])
            first[c] = t
            assert abs(mg[t]) < 2e-3, (c, t, mg[t])
    assert np.median(first) >= nmc // 2, sorted(first)
    whole = first == nmc
    rel = np.abs(ca[:K][whole] - oca[whole]) / np.maximum(np.abs(oca[whole]), 1.0)
    assert rel.max() < 1e-4, rel.max()
    print("\nmulti-lane FP64-decision kernel vs FP64 oracle: %d/%d chains follow all %d steps, others part at %s; "
          "estimates of followed chains max rel diff %.2e" % (whole.sum(), K, nmc, sorted(int(t) for t in first[~whole]),
                                                              rel.max()))


def test_lanes_analytic_moments():
    import mcintegratorplusplus_gb300 as mcig
    _, _, _, _, m1, m2 = mixture()
    exact = np.concatenate([[m2.sum()], m1, m2])
    nc = 4096
    r = run(mcig, mcig.PREC_FP32, 8, nc=nc, nmc=4096, f64=1, seed=5, moments=True)
    ca = r["ca"][:, :1 + 2 * NDIM]
    z = np.abs(ca.mean(0) - exact) / (ca.std(0, ddof=1) / np.sqrt(nc))
    assert z.max() < 3.5, z  # 65 moments: the largest of 65 normal deviates
    assert np.mean(z < 3.0) > 0.95
