"""Edge sizes of the path against the oracle and against itself.

* Dimensions at the ends of the device range, ndim 1 and 64 (the general kernel's maximum),
  with all-coordinate, single-coordinate vector and MultiStepMove moves: the FP64 kernel
  replaying the oracle's recorded draws reproduces the oracle's run (accept/reject counts,
  calibrated steps and walkers exactly, estimates within 1e-12), three chains at once.
* Chain counts that fill no whole block or warp (1, 37, 100): a chain's Philox stream does
  not depend on the launch, so chain c gives the same numbers bit for bit whatever the number
  of chains beside it, through the register-resident, the multi-lane and the general kernel.
* The smallest sample counts the estimators accept, and the errors below them.
"""
import numpy as np
import pytest

import cases
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _spec(ndim, move, veclen, seed, nmc, blocksize=16, estim=-1, obsset=0):
    return dict(name="edge", ndim=ndim, seed=seed, move=move, veclen=veclen, pdf=0, obsset=obsset,
                blocksize=blocksize, nskip=1, estim=estim, nfind=-50, ndecorr=300, nmc=nmc, periodic=0, target=0.5,
                nbits=nmc)


@pytest.mark.parametrize("ndim,move,veclen", [(1, 0, 0), (1, 2, 1), (64, 1, 0), (64, 2, 1), (64, 3, 0)])
def test_replay_at_dimension_limits(ndim, move, veclen):
    import mcintegratorplusplus_gb300 as mcig
    r = _spec(ndim, move, veclen, 900 + ndim + move, 2048)
    seeds = [11, 12, 13]
    o = orc.OracleMCI(ndim, len(seeds))
    cases.configure(o, r, lambda mm, s: mm.set_seeds(seeds))
    o.set_record(True)
    o.integrate(0, True, True)
    oavg, oerr, oca, oce = o.integrate(r["nmc"], False, False, per_chain=True)
    tape, lens = o.get_tapes()
    g = mcig.MCI(ndim, len(seeds), precision=mcig.PREC_FP64)
    cases.configure(g, r, lambda mm, s: None)
    g.setReplay(tape, lens)
    g.integrate(0, True, True)
    avg, err = g.integrate(r["nmc"], False, False)
    ca, ce = g.getChainResults()
    a, _ = g.getCounts()
    oa, _ = o.counts()
    np.testing.assert_array_equal(a, oa)
    np.testing.assert_array_equal(g.getX(), o.get_x())
    np.testing.assert_allclose(ca, oca, rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(ce, oce, rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(avg, oavg, rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(err, oerr, rtol=1e-12, atol=1e-300)


def _chains_run(mcig, nc, kernel, ndim=16, lanes=0):
    m = mcig.MCI(ndim, nc, precision=mcig.PREC_FP32)
    m.setSeed(4242)
    if ndim == 32:  # the multi-lane kernel's mixture
        rng = np.random.default_rng(8)
        ncomp = 4
        w = rng.dirichlet(np.ones(ncomp))
        means = rng.standard_normal((ncomp, ndim))
        widths = 10.0 ** rng.uniform(-0.3, 0.3, (ncomp, ndim))
        m.addSamplingFunction(mcig.PDF_GAUSS_MIX, np.concatenate([[ncomp], w, means.ravel(), widths.ravel()]))
    else:
        m.addSamplingFunction(mcig.PDF_GAUSS)
    m.setTrialMove(mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
    m.setNdecorrelationSteps(200)
    m.addObservable(mcig.OBS_X2SUM, (), 32, 1, False, mcig.EST_UNCORRELATED)
    m.addObservable(mcig.OBS_XND, (), 1, 1, False, mcig.EST_UNCORRELATED)
    if lanes:
        m.setLanes(lanes)
    m.setKernel(kernel)
    m.integrate(1024)
    ca, ce = m.getChainResults()
    return dict(ca=ca, ce=ce, x=m.getX(), steps=m.getMRT2Steps(), ctr=m.getStepCounters(), acc=m.getCounts()[0])


@pytest.mark.parametrize("kernel,ndim,lanes", [(2, 16, 0), (1, 16, 0), (3, 32, 8)])
def test_chain_results_do_not_depend_on_the_chain_count(kernel, ndim, lanes):
    import mcintegratorplusplus_gb300 as mcig
    ref = _chains_run(mcig, 100, kernel, ndim, lanes)
    for nc in (1, 37):
        r = _chains_run(mcig, nc, kernel, ndim, lanes)
        for k in ref:
            np.testing.assert_array_equal(r[k], ref[k][:nc], err_msg="%s, %d chains" % (k, nc))


def test_smallest_sample_counts_and_errors_below_them():
    import mcintegratorplusplus_gb300 as mcig
    m = mcig.MCI(3, 4, precision=mcig.PREC_FP64)
    m.setSeed(5)
    m.addSamplingFunction(mcig.PDF_GAUSS)
    m.setNdecorrelationSteps(0)
    m.setNfindMRT2Iterations(0)
    m.addObservable(mcig.OBS_X2SUM, (), 1, 1, False, mcig.EST_UNCORRELATED)  # Full, n >= 2
    avg, err = m.integrate(2)
    assert np.all(np.isfinite(avg)) and np.all(np.isfinite(err))
    with pytest.raises(ValueError, match="larger than 1"):
        m.integrate(1)
    m.popObservable()
    m.addObservable(mcig.OBS_X2SUM, (), 1, 1, False, mcig.EST_FCBLOCKER)  # Full, n >= 50
    m.integrate(50)
    with pytest.raises(ValueError, match="50"):
        m.integrate(49)
    m.popObservable()
    m.addObservable(mcig.OBS_X2SUM, (), 1, 1, False, mcig.EST_MJBLOCKER)  # Full, a power of two
    m.integrate(64)
    with pytest.raises(ValueError, match="power of two"):
        m.integrate(48)
