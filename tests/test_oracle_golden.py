"""Pin the CPU oracle against the reference's own outputs (tests/golden/reference_golden.json,
generated by tests/golden/make_golden.py from the reference compiled from its sources)."""
import numpy as np
import pytest

from oracle import oracle as orc
import cases


G = cases.golden()


def test_mt19937_64_known_answers():
    # C++ [rand.predef]: the 10000th output of a default-seeded (5489) mt19937_64
    assert int(orc.mt64_stream(5489, 10000)[-1]) == 9981545732273789042
    ref = [int(v) for v in G["mt64_seed1234"]]
    assert [int(v) for v in orc.mt64_stream(1234, 8)] == ref


def test_distributions_match_libstdcxx():
    assert list(orc.canonical_stream(1234, 8)) == G["canonical_seed1234"]
    assert list(orc.normal_stream(1234, 9)) == G["normal_seed1234"]
    assert list(orc.uniform_int_stream(1234, 16, 3)) == [int(v) for v in G["uniform_int3_seed1234"]]


@pytest.mark.parametrize("srrd", range(2, 10))
def test_other_move_distributions_match_libstdcxx(srrd):
    """Student t, Cauchy and the symmetrized exponential, gamma, Weibull, lognormal,
    chi-squared and Fisher distributions of the reference's moves: 64 draws of each, bit for
    bit (they drive the reference's SRRD moves; the tape carries them to the device)."""
    g = cases.golden()
    np.testing.assert_array_equal(orc.srrd_stream(srrd, 1234, 64), np.array(g["srrd%d_seed1234" % srrd]))


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10
    assert orc.philox4x32_10([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert orc.philox4x32_10([0xffffffff] * 4, [0xffffffff] * 2) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6,
                                                                    0x6d5451fd]
    assert orc.philox4x32_10([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


@pytest.fixture(scope="module")
def series():
    s = G["series"]
    return orc.splitmix64_ar1(s["seed"], s["n"], s["ndim"], s["phi"])


def test_estimators_match_reference(series):
    x = series
    for est, key in ((cases.EST_UNCORRELATED, "est_uncorr"), (cases.EST_FCBLOCKER, "est_fc"),
                     (cases.EST_MJBLOCKER, "est_mj")):
        a, e = orc.estimate(est, x)
        assert list(a) == G[key + "_avg"], key
        assert list(e) == G[key + "_err"], key
    a, e = orc.block_estimate(x, 2048)
    assert list(a) == G["est_block2048_avg"] and list(e) == G["est_block2048_err"]
    a, e = orc.estimate(cases.EST_FCBLOCKER, x[:, 0].copy())
    assert list(a) == G["est_fc1d"] and list(e) == G["est_fc1d_err"]
    a, e = orc.estimate(cases.EST_MJBLOCKER, x[:, 0].copy())
    assert list(a) == G["est_mj1d"] and list(e) == G["est_mj1d_err"]
    a, e = orc.estimate(cases.EST_CORRELATED, x[:10000])
    assert list(a) == G["est_corr10000_avg"] and list(e) == G["est_corr10000_err"]
    y = orc.splitmix64_ar1(7, 4096, 17, 0.5)
    a, e = orc.estimate(cases.EST_MJBLOCKER, y)
    assert list(a) == G["est_mj17_avg"] and list(e) == G["est_mj17_err"]
    a, e = orc.estimate(cases.EST_FCBLOCKER, y)
    assert list(a) == G["est_fc17_avg"] and list(e) == G["est_fc17_err"]


def test_estimator_errors():
    with pytest.raises(orc.OracleError):
        orc.estimate(cases.EST_MJBLOCKER, np.zeros((3000, 1)))  # not a power of two
    with pytest.raises(orc.OracleError):
        orc.estimate(cases.EST_FCBLOCKER, np.zeros((49, 1)))  # fewer than 50 samples
    with pytest.raises(orc.OracleError):
        orc.estimate(cases.EST_UNCORRELATED, np.zeros((1, 2)))
    # constant data: every MJBlocker level fails its test; the last level is used (error 0)
    a, e = orc.estimate(cases.EST_MJBLOCKER, np.full((1024, 2), 1.25))
    assert list(a) == [1.25, 1.25] and list(e) == [0.0, 0.0]


def test_accumulators_match_reference():
    w = G["walk"]
    xs, acc = orc.splitmix64_walk(w["seed"], w["accept_seed"], w["n"], w["ndim"], w["phi"])
    for key, bs, skip in (("acc_simple_1", 0, 1), ("acc_simple_2", 0, 2), ("acc_block16_1", 16, 1),
                          ("acc_block8_2", 8, 2), ("acc_full_1", 1, 1), ("acc_full_3", 1, 3)):
        d = orc.accumulate_walk(cases.OBS_XND, xs, acc, bs, skip)
        assert list(d) == G[key], key


def _oracle_run(r, record=False):
    m = orc.OracleMCI(r["ndim"], 1)
    cases.configure(m, r, lambda mm, s: mm.set_seeds([s]))
    if record:
        m.set_record(True)
    m.integrate(0, True, True)
    step = [m.get_mrt2step(0, i) for i in range(len(G[r["name"]]["step"]))]
    xstart = m.get_x()[0].copy()
    acc_burn = m.acceptance_rate()
    avg, err = m.integrate(r["nmc"], False, False)
    return m, avg, err, step, xstart, acc_burn


@pytest.mark.parametrize("name", [r["name"] for r in cases.runs()])
def test_integration_matches_reference(name):
    r = cases.run(name)
    g = G[name]
    m, avg, err, step, xstart, acc_burn = _oracle_run(r, record=True)
    assert step == g["step"]
    assert list(xstart) == g["xstart"]
    assert acc_burn == g["acc_burn"]
    assert list(avg) == g["avg"]
    assert list(err) == g["err"]
    assert list(m.get_x()[0]) == g["xend"]
    assert m.acceptance_rate() == g["acc_main"]
    bits, start = m.get_accept_bits(0)
    ref_bits = cases.unpack_bits(g["bits"], g["nbits"])
    assert list(bits[start:start + g["nbits"]]) == ref_bits


def test_tape_replay_reproduces_run():
    """Replaying the recorded draws (the device replay input) reproduces the run exactly."""
    r = cases.run("multistep_exp")
    m, avg, err, *_ = _oracle_run(r, record=True)
    tape, lens = m.get_tapes()
    m2 = orc.OracleMCI(r["ndim"], 1)
    cases.configure(m2, r, lambda mm, s: mm.set_seeds([s + 1]))  # wrong seed: the tape must decide
    m2.set_replay(tape, lens)
    m2.integrate(0, True, True)
    avg2, err2 = m2.integrate(r["nmc"], False, False)
    assert list(avg2) == list(avg) and list(err2) == list(err)


def test_multichain_mpimci_reduction():
    """Several chains combine with the MPIMCI formula (src/MPIMCI.cpp:85-92)."""
    r = cases.run("all_gauss_block")
    per = []
    for s in (11, 12, 13):
        m = orc.OracleMCI(3, 1)
        cases.configure(m, r, lambda mm, _s: mm.set_seeds([s]))
        m.integrate(0, True, True)
        per.append(m.integrate(4096, False, False))
    mm = orc.OracleMCI(3, 3)
    cases.configure(mm, r, lambda x, _s: x.set_seeds([11, 12, 13]))
    mm.integrate(0, True, True)
    avg, err = mm.integrate(4096, False, False, nthreads=3)
    a = np.array([p[0] for p in per])
    e = np.array([p[1] for p in per])
    np.testing.assert_allclose(avg, a.sum(0) / 3, rtol=1e-15)
    np.testing.assert_allclose(err, np.sqrt((e * e).sum(0)) / 3, rtol=1e-15)


def test_error_behaviour():
    m = orc.OracleMCI(3, 1)
    m.add_observable(cases.OBS_X2SUM)
    with pytest.raises(orc.OracleError, match="infinite domain"):
        m.integrate(100)
    m.add_sampling_function(cases.PDF_GAUSS)
    m.clear_observables()
    m.add_observable(cases.OBS_X2SUM, (), 3, 1)  # 100 accumulations are not a multiple of 3
    with pytest.raises(orc.OracleError, match="multiple of the requested block size"):
        m.integrate(100, False, False)
    with pytest.raises(orc.OracleError, match="equilibration"):
        m.add_observable(cases.OBS_X2SUM, (), 0, 1, True, cases.EST_NOOP)
    with pytest.raises(orc.OracleError, match="multiple of passed veclen"):
        m.set_trial_move(cases.MOVE_VEC, 0, 2)


def test_oracle_logpdf_observable_is_minus_the_protos():
    """The log-pdf observable of the oracle (a dependent observable) equals -sum of the
    Gauss protos x_i^2 of the recorded walker, summed in index order."""
    from oracle import oracle as orc
    m = orc.OracleMCI(3, 1)
    m.set_seeds([11])
    m.add_sampling_function(1, ())          # Gauss: exp(-sum x_i^2)
    m.add_observable(1, (), 1, 1)            # x_i, Full
    m.add_observable(9, (), 1, 1)            # log pdf, Full
    m.integrate(0, True, True)
    m.integrate(64, False, False)
    xs = m.obs_data(0).reshape(64, 3)
    lp = m.obs_data(1).reshape(64)
    for x, v in zip(xs, lp):
        s = 0.
        for xi in x:
            s = s + xi * xi
        assert v == 0. - s
