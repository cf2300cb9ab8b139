"""The register-resident float kernels (mcig_fast_kernel, mcig_calib_kernel) on the 16-D
correlated-Gaussian workload (65,536-chain benchmark configuration: dense precision matrix,
Gaussian all-coordinate move, automatic per-chain step calibration, 1,000 burn-in steps,
x.x and x_i in Block and Full accumulators), checked against the FP64 oracle driven by the
kernel's own Philox draws.

The oracle (the reference's algorithm in double, reference operation order) draws from the
same Philox counters as the device chain (orc_set_philox, layout 1: the float kernels' draws
evaluated in double), so a device chain and its oracle chain take the same decisions until
a step whose acceptance margin log(u) - log(a) lies within the float kernel's rounding of
zero.  Each phase (calibration, burn-in, sampling) restarts the oracle from the device's
state at the phase start (walker, step size, Philox counter), so float rounding cannot
accumulate across phases.  Checked per chain:
  * calibration and burn-in: the end state equals the oracle's (steps to float rounding,
    counters exactly), or the oracle's record holds a near-tie that explains the difference;
  * sampling: the walker of every step (the Full x_i samples) equals the oracle's until the
    first step where they part, and at that step the oracle's margin is a near-tie;
  * estimates: per chain, the float result against the FP64 result on the same draws.
Reference: MCI::findMRT2Step / doStepMRT2 / sample (src/MCIntegrator.cpp:87-168, 290-360).
"""
import numpy as np
import pytest

from oracle import oracle as orc

NDIM = 16
SEED = 20241203
NMC = 10000
BURNIN = 1000
NBLOCKS = 100
K_ORACLE = 48          # chains replayed by the oracle
NEAR_TIE = 2e-3        # |log u - log a| below which float and double may decide apart
X_PART = 1e-2          # walkers this far apart have taken different decisions


def target(seed=2024):
    rng = np.random.default_rng(seed)
    Q, R = np.linalg.qr(rng.standard_normal((NDIM, NDIM)))
    Q = Q * np.sign(np.diag(R))
    lam = 10.0 ** rng.uniform(-1.0, 1.0, NDIM)
    Sigma = Q @ np.diag(lam) @ Q.T
    P = Q @ np.diag(1.0 / lam) @ Q.T
    return Sigma, 0.5 * (P + P.T)


def configure(m, P, nmc=NMC, nblocks=NBLOCKS):
    m.add_sampling_function(3, P)            # GAUSS_PREC
    m.set_trial_move(0, 1, 0)                # all-coordinate, Gaussian
    m.set_nfind_mrt2_iterations(-50)
    m.set_ndecorrelation_steps(BURNIN)
    bs = nmc // nblocks
    m.add_observable(0, (), bs, 1, False, 1)  # x.x, Block, Uncorrelated
    m.add_observable(1, (), bs, 1, False, 1)  # x_i, Block, Uncorrelated
    m.add_observable(0, (), 1, 1, False, 1)   # x.x, Full
    m.add_observable(1, (), 1, 1, False, 1)   # x_i, Full


def _oracle_from(state, P, k, nthreads=8):
    """Oracle chains 0..k-1 at the device state (walker, steps, counters)."""
    o = orc.OracleMCI(NDIM, k)
    configure(o, P)
    o.set_x(state["x"][:k])
    o.set_chain_steps(state["steps"][:k])
    o.set_philox(SEED, 0, state["ctr"][:k], layout=1)
    o.set_record(True)
    return o


def _device_state(m):
    return {"x": m.getX(), "steps": m.getMRT2Steps(), "ctr": m.getStepCounters().astype(np.uint64)}


def _min_abs_margin(o, c, lo=0, hi=None):
    mg = o.get_margins(c)
    mg = mg[lo:hi]
    return float(np.min(np.abs(mg))) if mg.size else np.inf


@pytest.mark.gpu
@pytest.mark.parametrize("prec_name,split", [("fp32", True), ("fp32_acc64", True), ("fp32", False)])
def test_fast_kernel_against_fp64_oracle_same_draws(prec_name, split):
    import mcintegratorplusplus_gb300 as mcig
    prec = {"fp32": mcig.PREC_FP32, "fp32_acc64": mcig.PREC_FP32_ACC64}[prec_name]
    Sigma, P = target()
    nc = 256
    m = mcig.MCI(NDIM, nc, device=0, precision=prec)
    m.setKernel(2)                 # the register-resident kernels only (error if not served)
    m.setCalibrationSplit(split)
    m.setSeed(SEED)
    m.setFullStorage(32)
    configure(m, P)
    s0 = _device_state(m)
    assert np.all(s0["ctr"] == 0) and np.allclose(s0["steps"], 0.05)

    # --- phase 1: findMRT2Step from x = 0, step 0.05, counter 0
    m.integrate(0, True, False)
    s1 = _device_state(m)
    o = _oracle_from(s0, P, K_ORACLE)
    o.integrate(0, True, False, nthreads=8)
    ostep = np.array([o.get_mrt2step(c) for c in range(K_ORACLE)])
    octr = o.philox_counters()
    same = (octr == s1["ctr"][:K_ORACLE]) & (np.abs(ostep / s1["steps"][:K_ORACLE, 0] - 1) < 1e-5)
    for c in np.nonzero(~same)[0]:  # a calibration that parted must contain a near-tie
        assert _min_abs_margin(o, c) < NEAR_TIE, (c, ostep[c], s1["steps"][c], octr[c], s1["ctr"][c])
    assert same.mean() >= 0.75, same.mean()
    # the float kernel's step is the double step rounded to float
    np.testing.assert_allclose(s1["steps"][:K_ORACLE, 0][same], ostep[same], rtol=1e-5)

    # --- phase 2: 1,000 burn-in steps from the device's calibrated state
    m.integrate(0, False, True)
    s2 = _device_state(m)
    o = _oracle_from(s1, P, K_ORACLE)
    o.integrate(0, False, True, nthreads=8)
    ox = o.get_x()
    assert np.array_equal(o.philox_counters(), s2["ctr"][:K_ORACLE])
    dx = np.max(np.abs(ox - s2["x"][:K_ORACLE]), axis=1)
    for c in np.nonzero(dx > X_PART)[0]:
        assert _min_abs_margin(o, c) < NEAR_TIE, (c, dx[c])
    assert np.mean(dx <= 1e-4) >= 0.9, np.sort(dx)[-8:]

    # --- phase 3: sampling with the four accumulators from the device's burnt-in state
    avg, err = m.integrate(NMC, False, False)
    ca, ce = m.getChainResults()
    o = _oracle_from(s2, P, K_ORACLE)
    oavg, oerr, oca, oce = o.integrate(NMC, False, False, nthreads=8, per_chain=True)
    xs_dev = m.getObsDataChains(3, 0, K_ORACLE).reshape(K_ORACLE, NMC, NDIM)
    xs_orc = o.obs_data(3).reshape(K_ORACLE, NMC, NDIM)
    first_part = np.full(K_ORACLE, NMC)
    for c in range(K_ORACLE):
        bits, start = o.get_accept_bits(c)
        mg = o.get_margins(c)[start:start + NMC]
        d = np.max(np.abs(xs_dev[c] - xs_orc[c]), axis=1)
        apart = np.nonzero(d > X_PART)[0]
        if apart.size:
            t = int(apart[0])
            first_part[c] = t
            assert abs(mg[t]) < NEAR_TIE, (c, t, mg[t])
            # before that step the float walker follows the double walker to rounding
            if t > 0:
                assert np.max(d[:t]) < 1e-3, (c, t, np.max(d[:t]))
        else:
            assert np.max(d) < 1e-3
    # most chains follow the oracle for most of the 10,000 steps
    assert np.median(first_part) >= 2000, np.sort(first_part)
    # estimates of chains that never parted: float against FP64 on the same draws
    whole = first_part == NMC
    if whole.any():
        rel = np.abs(ca[:K_ORACLE][whole] - oca[whole]) / np.maximum(np.abs(oca[whole]), 1.0)
        assert rel.max() < 1e-4, rel.max()
    # combined over the oracle's chains: the float result against the FP64 one, in units of
    # the standard error from the spread of the chain means (the chains that part become
    # independent samples of the same target, the others agree to float rounding)
    dev_k = ca[:K_ORACLE].mean(0)
    orc_k = oca.mean(0)
    sem_k = oca.std(0, ddof=1) / np.sqrt(K_ORACLE)
    zk = np.abs(dev_k - orc_k) / sem_k
    assert zk.max() < 3.0, zk
    print("\nfloat kernel vs FP64 oracle (%s, split %s): calibration identical %d/%d, burn-in identical %d/%d, "
          "sampling: %d/%d chains follow all %d steps, first parting step of the others %s, "
          "per-chain estimates of followed chains max rel diff %.2e, combined |f32 - f64| / sem max %.3f"
          % (prec_name, split, same.sum(), K_ORACLE, int(np.sum(dx <= 1e-4)), K_ORACLE, int(whole.sum()), K_ORACLE,
             NMC, sorted(int(t) for t in first_part[~whole]), rel.max() if whole.any() else float("nan"), zk.max()))

    # --- (b) the whole 256-chain run against the analytic target: x.x -> tr Sigma, x_i -> 0,
    # errors from the spread of the chain means (chains are independent)
    sem = ca.std(0, ddof=1) / np.sqrt(nc)
    exact = np.concatenate([[np.trace(Sigma)], np.zeros(NDIM)])
    z = np.abs(ca.mean(0)[:NDIM + 1] - exact) / sem[:NDIM + 1]
    assert z.max() < 3.5, z


@pytest.mark.gpu
def test_fast_kernel_c2_analytic_4096_chains():
    """4,096 chains of the benchmark configuration: x.x within 3 combined standard errors of
    tr Sigma and every coordinate mean within 3 of 0, the standard error from the spread of
    the chain means (each chain's own block error underestimates it: tau_int of x.x is
    about 230 steps, longer than the 100-step blocks)."""
    import mcintegratorplusplus_gb300 as mcig
    Sigma, P = target()
    nc = 4096
    for prec in (mcig.PREC_FP32, mcig.PREC_FP32_ACC64):
        m = mcig.MCI(NDIM, nc, device=0, precision=prec)
        m.setKernel(2)
        m.setSeed(SEED + 1)
        m.setFullStorage(32)
        configure(m, P)
        avg, err = m.integrate(NMC)
        ca, ce = m.getChainResults()
        sem = ca.std(0, ddof=1) / np.sqrt(nc)
        exact = np.concatenate([[np.trace(Sigma)], np.zeros(NDIM)])
        for off in (0, NDIM + 1):  # Block and Full copies
            z = np.abs(ca.mean(0)[off:off + NDIM + 1] - exact) / sem[off:off + NDIM + 1]
            assert z.max() < 3.0, (prec, off, z)
        # Block and Full give the same chain means (same samples, different sums)
        np.testing.assert_allclose(ca[:, :NDIM + 1], ca[:, NDIM + 1:], rtol=2e-5, atol=2e-5)
