"""Parity of the device path with the oracle (and through it with the reference).

* replay: the device consumes the draws the reference consumed (recorded by the
  oracle, which is pinned bit-exact to the reference in test_oracle_golden.py)
  and must reproduce the accept/reject sequence bit-exactly, the estimates
  within 1e-12 relative, the step sizes and final walker exactly;
* estimators and accumulators on identical arrays: within 1e-12 relative;
* Philox runs: known-answer vectors and 3-sigma statistical agreement.
"""
import numpy as np
import pytest

import cases
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

G = cases.golden()
RTOL = 1e-12


@pytest.fixture(scope="module")
def mcig():
    import mcintegratorplusplus_gb300 as m
    m._lib.load()
    return m


def test_philox_known_answers(mcig):
    for ctr, key in (([0, 0, 0, 0], [0, 0]), ([0xffffffff] * 4, [0xffffffff] * 2),
                     ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]),
                     ([7, 1, 12345, 0x10001], [0xdeadbeef, 42])):
        assert mcig.philox_block(ctr, key) == orc.philox4x32_10(ctr, key)


def _oracle_recorded(r):
    m = orc.OracleMCI(r["ndim"], 1)
    cases.configure(m, r, lambda mm, s: mm.set_seeds([s]))
    m.set_record(True)
    m.integrate(0, True, True)
    avg, err = m.integrate(r["nmc"], False, False)
    tape, lens = m.get_tapes()
    bits, start = m.get_accept_bits(0)
    steps = [m.get_mrt2step(0, i) for i in range(len(G[r["name"]]["step"]))]
    return dict(avg=avg, err=err, tape=tape, lens=lens, bits=bits[start:], steps=steps, x=m.get_x()[0],
                rate=m.acceptance_rate(), counts=m.counts())


REPLAY_CASES = [r["name"] for r in cases.runs() if r["nmc"] <= (1 << 20)]


@pytest.mark.parametrize("name", REPLAY_CASES)
def test_replay_reproduces_reference_run(mcig, name):
    r = cases.run(name)
    ref = _oracle_recorded(r)
    g = mcig.MCI(r["ndim"], 1, precision=mcig.PREC_FP64)
    cases.configure(g, r, lambda mm, s: mm.set_seeds([s]))
    g.setReplay(ref["tape"], ref["lens"])
    g.setRecordAccepts(True)
    g.integrate(0, True, True)
    avg, err = g.integrate(r["nmc"], False, False)
    bits = g.getAcceptBits()[:, 0]
    # accept/reject sequence and counts: bit-exact
    assert bits.shape[0] == r["nmc"]
    mism = np.nonzero(bits != ref["bits"][:r["nmc"]])[0]
    assert mism.size == 0, "first mismatch at step %d" % (mism[0] if mism.size else -1)
    a, rj = g.getCounts()
    assert (a[0], rj[0]) == (ref["counts"][0][0], ref["counts"][1][0])
    assert g.getAcceptanceRate() == ref["rate"]
    # calibrated step sizes and final walker: exact
    assert [g.getMRT2Step(i) for i in range(len(ref["steps"]))] == ref["steps"]
    np.testing.assert_array_equal(g.getX()[0], ref["x"])
    # estimates within 1e-12 relative
    np.testing.assert_allclose(avg, ref["avg"], rtol=RTOL, atol=1e-300)
    np.testing.assert_allclose(err, ref["err"], rtol=RTOL, atol=1e-300)
    # and the reference's own golden numbers
    np.testing.assert_allclose(avg, G[name]["avg"], rtol=RTOL)
    np.testing.assert_allclose(err, G[name]["err"], rtol=RTOL)


def test_replay_multichain_matches_oracle(mcig):
    """Four chains, each replaying its own reference stream, combined with the MPIMCI formula."""
    r = cases.run("all_gauss_block")
    seeds = [3, 5, 7, 11]
    m = orc.OracleMCI(3, len(seeds))
    cases.configure(m, r, lambda mm, s: mm.set_seeds(seeds))
    m.set_record(True)
    m.integrate(0, True, True)
    avg, err, ca, ce = m.integrate(8192, False, False, per_chain=True)
    tape, lens = m.get_tapes()
    g = mcig.MCI(3, len(seeds), precision=mcig.PREC_FP64)
    cases.configure(g, r, lambda mm, s: None)
    g.setReplay(tape, lens)
    g.integrate(0, True, True)
    gavg, gerr = g.integrate(8192, False, False)
    gca, gce = g.getChainResults()
    np.testing.assert_allclose(gca, ca, rtol=RTOL)
    np.testing.assert_allclose(gce, ce, rtol=RTOL)
    np.testing.assert_allclose(gavg, avg, rtol=RTOL)
    np.testing.assert_allclose(gerr, err, rtol=RTOL)
    a, _ = g.getCounts()
    oa, _ = m.counts()
    np.testing.assert_array_equal(a, oa)


def test_replay_obs_data_matches_oracle(mcig):
    """Raw accumulator arrays (Full and Block) equal the oracle's."""
    r = dict(cases.run("typed_all"))
    ref = orc.OracleMCI(3, 1)
    cases.configure(ref, r, lambda mm, s: mm.set_seeds([s]))
    ref.add_observable(cases.OBS_XND, (), 1, 2)
    ref.add_observable(cases.OBS_LOGPDF, (), 1, 1)  # depends on the sampling functions
    ref.set_record(True)
    ref.integrate(0, True, True)
    ref.integrate(4096, False, False)
    tape, lens = ref.get_tapes()
    g = mcig.MCI(3, 1, precision=mcig.PREC_FP64)
    cases.configure(g, r, lambda mm, s: None)
    g.add_observable(cases.OBS_XND, (), 1, 2)
    g.add_observable(cases.OBS_LOGPDF, (), 1, 1)
    g.setReplay(tape, lens)
    g.integrate(0, True, True)
    g.integrate(4096, False, False)
    for o in range(4):
        np.testing.assert_array_equal(g.getObsData(o), ref.obs_data(o))


@pytest.fixture(scope="module")
def series():
    s = G["series"]
    return orc.splitmix64_ar1(s["seed"], s["n"], s["ndim"], s["phi"])


def test_estimators_on_identical_arrays(mcig, series):
    x = series
    y = orc.splitmix64_ar1(7, 4096, 17, 0.5)
    for est in (cases.EST_UNCORRELATED, cases.EST_FCBLOCKER, cases.EST_MJBLOCKER, cases.EST_CORRELATED,
                cases.EST_NOOP):
        for arr in (x, x[:, 0].copy(), x[:10000] if est != cases.EST_MJBLOCKER else x[:8192], y):
            a, e = mcig.estimate(est, arr)
            oa, oe = orc.estimate(est, arr)
            np.testing.assert_allclose(a, oa, rtol=RTOL, atol=0)
            np.testing.assert_allclose(e, oe, rtol=RTOL, atol=0)
    a, e = mcig.estimate(cases.EST_MJBLOCKER, x)
    np.testing.assert_allclose(a, G["est_mj_avg"], rtol=RTOL)
    np.testing.assert_allclose(e, G["est_mj_err"], rtol=RTOL)
    a, e = mcig.estimate(cases.EST_FCBLOCKER, x)
    np.testing.assert_allclose(e, G["est_fc_err"], rtol=RTOL)


def test_estimator_edge_cases(mcig):
    with pytest.raises(ValueError, match="power of two"):
        mcig.estimate(cases.EST_MJBLOCKER, np.zeros((3000, 1)))
    with pytest.raises(ValueError):
        mcig.estimate(cases.EST_FCBLOCKER, np.zeros((49, 2)))
    with pytest.raises(ValueError):
        mcig.estimate(cases.EST_UNCORRELATED, np.zeros((1, 2)))
    a, e = mcig.estimate(cases.EST_MJBLOCKER, np.full((1024, 2), 1.25))  # constant data
    assert list(a) == [1.25, 1.25] and list(e) == [0.0, 0.0]
    a, e = mcig.estimate(cases.EST_MJBLOCKER, np.array([[2.5]]))  # n = 1: no level
    assert list(a) == [2.5] and list(e) == [0.0]


def test_accumulators_on_recorded_walk(mcig):
    w = G["walk"]
    xs, acc = orc.splitmix64_walk(w["seed"], w["accept_seed"], w["n"], w["ndim"], w["phi"])
    for key, bs, skip in (("acc_simple_1", 0, 1), ("acc_simple_2", 0, 2), ("acc_block16_1", 16, 1),
                          ("acc_block8_2", 8, 2), ("acc_full_1", 1, 1), ("acc_full_3", 1, 3)):
        d = mcig.accumulate_walk(cases.OBS_XND, xs, acc, bs, skip)
        np.testing.assert_allclose(d, G[key], rtol=RTOL, atol=0)
        np.testing.assert_allclose(d, orc.accumulate_walk(cases.OBS_XND, xs, acc, bs, skip), rtol=RTOL, atol=0)
    with pytest.raises(ValueError, match="multiple of the requested block size"):
        mcig.accumulate_walk(cases.OBS_XND, xs[:100], acc[:100], 3, 1)


def _c1(mcig, nchains, prec, seed=1234, nmc=1 << 14):
    g = mcig.MCI(3, nchains, precision=prec)
    g.setSeed(seed)
    g.addSamplingFunction(mcig.PDF_GAUSS)
    g.setNdecorrelationSteps(1000)
    g.addObservable(mcig.OBS_X2SUM, (), 1024, 1, True, mcig.EST_MJBLOCKER)
    g.addObservable(mcig.OBS_XND, (), 1024, 1, True, mcig.EST_MJBLOCKER)
    avg, err = g.integrate(nmc)
    return g, avg, err


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_philox_statistics_c1(mcig, prec):
    """exp(-x.x) in 3-D: <x.x> = 1.5, <x_i> = 0, within 3 sigma; acceptance near the 0.5 target."""
    g, avg, err = _c1(mcig, 1024, prec)
    z = np.abs(avg - np.array([1.5, 0, 0, 0])) / err
    assert np.all(z < 3.5), (avg, err)
    assert 0.4 < g.getAcceptanceRate() < 0.6
    steps = g.getMRT2Steps()
    assert np.all(np.abs(steps - 1.09) < 0.4)


def test_philox_agrees_with_reference_run(mcig):
    """GPU Philox chains vs the reference's own C1 result (seed 1234, 2^20 steps) within 3 combined sigma."""
    g, avg, err = _c1(mcig, 256, 1, seed=99, nmc=1 << 14)
    ref_avg = np.array(G["c1_seed1234"]["avg"])
    ref_err = np.array(G["c1_seed1234"]["err"])
    z = np.abs(avg - ref_avg) / np.sqrt(err ** 2 + ref_err ** 2)
    assert np.all(z < 3.5), z


def test_philox_runs_are_reproducible_and_resume(mcig):
    g1, a1, e1 = _c1(mcig, 64, 1, seed=5)
    g2, a2, e2 = _c1(mcig, 64, 1, seed=5)
    np.testing.assert_array_equal(a1, a2)
    a3, _ = g1.integrate(1 << 12, False, False)  # continues the chain: different numbers
    assert not np.array_equal(a3, a1)


def test_vec_and_multistep_moves_statistics(mcig):
    for setup in ("vec", "multistep", "gauss"):
        g = mcig.MCI(3, 512, precision=mcig.PREC_FP32)
        g.setSeed(17)
        g.addSamplingFunction(mcig.PDF_GAUSS)
        if setup == "vec":
            g.setTrialMove(mcig.MOVE_VEC, mcig.SRRD_UNIFORM, 1)
        elif setup == "multistep":
            g.setMultiStepMove(3, mcig.SRRD_UNIFORM, 1, 0.1)
            g.addMultiStepSamplingFunction(mcig.PDF_EXP)
            g.setTargetAcceptanceRate(0.85)
        else:
            g.setTrialMove(mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
        g.setNdecorrelationSteps(1000)
        g.addObservable(mcig.OBS_X2MEAN, (), 1, 1)
        g.addObservable(mcig.OBS_X2, (), 1, 1)
        avg, err = g.integrate(8192)
        z = np.abs(avg - 0.5) / err
        assert np.all(z < 3.5), (setup, avg, err)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_every_srrd_distribution_statistics(mcig, prec):
    """All ten SRRDType distributions (Factories.hpp:119-133) as all-coordinate and
    vector moves (and as MultiStepMove sub-moves) sample exp(-x.x): <x_i^2> = 1/2."""
    p = mcig.PREC_FP64 if prec == "fp64" else mcig.PREC_FP32
    for srrd in range(10):
        for mode in ("all", "vec", "multistep"):
            g = mcig.MCI(4, 256, precision=p)
            g.setSeed(100 + srrd)
            g.addSamplingFunction(mcig.PDF_GAUSS)
            if mode == "all":
                g.setTrialMove(mcig.MOVE_ALL, srrd)
            elif mode == "vec":
                g.setTrialMove(mcig.MOVE_VEC, srrd, 2)
            else:
                g.setMultiStepMove(2, srrd, 1, 0.3)
                g.addMultiStepSamplingFunction(mcig.PDF_EXP)
                g.setNfindMRT2Iterations(0)
            g.setNdecorrelationSteps(500)
            g.addObservable(mcig.OBS_X2, (), 256, 1, False, mcig.EST_UNCORRELATED)
            avg, err = g.integrate(1 << 14)
            z = np.abs(avg - 0.5) / err
            assert np.all(z < 4.0), (srrd, mode, avg, err)
            assert 0.05 < g.getAcceptanceRate() <= 1.0, (srrd, mode)


def test_periodic_and_no_pdf_paths(mcig):
    g = mcig.MCI(3, 256, precision=mcig.PREC_FP64)
    g.setSeed(3)
    g.setIRange(-5.0, 5.0)
    g.addObservable(mcig.OBS_GAUSSX2, (), 1, 1, False, False)
    avg, err = g.integrate(10000, False, False)
    assert abs(avg[0] - 0.5) < 3.5 * err[0]
    x = g.getX()
    assert np.all(x >= -5.0) and np.all(x <= 5.0)


def test_error_behaviour(mcig):
    g = mcig.MCI(3, 4)
    g.addObservable(mcig.OBS_X2SUM)
    with pytest.raises(mcig.DomainError, match="infinite domain"):
        g.integrate(100)
    g.addSamplingFunction(mcig.PDF_GAUSS)
    g.clearObservables()
    g.addObservable(mcig.OBS_X2SUM, (), 3, 1)
    with pytest.raises(ValueError, match="multiple of the requested block size"):
        g.integrate(100, False, False)
    with pytest.raises(ValueError, match="equilibration"):
        g.addObservable(mcig.OBS_X2SUM, (), 0, 1, True, mcig.EST_NOOP)
    with pytest.raises(ValueError, match="multiple of passed veclen"):
        g.setTrialMove(mcig.MOVE_VEC, 0, 2)
    with pytest.raises(mcig.DomainError, match="Unhandled SRRDType"):
        g.setTrialMove(mcig.MOVE_ALL, 10)
    with pytest.raises(ValueError):
        g.addSamplingFunction(mcig.PDF_GAUSS_PREC, np.eye(2))
    g2 = mcig.MCI(3, 1, precision=mcig.PREC_FP64)
    g2.addSamplingFunction(mcig.PDF_GAUSS)
    g2.addObservable(mcig.OBS_X2SUM)
    g2.setReplay(np.full(10, 0.5))
    with pytest.raises(RuntimeError, match="tape exhausted"):
        g2.integrate(100, False, False)
