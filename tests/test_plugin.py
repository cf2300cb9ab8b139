"""User functors compiled as a plugin (include/mcig/plugin.cuh, tests/plugins/gauss_plugin.cu):
the plugin builds and loads; integrals with its functors equal integrals with the built-in kinds
of the same arithmetic bit for bit (double path), reproduce the oracle's run under replay, and
agree statistically on the float paths; what the plugin kernel does not serve is an error."""
import ctypes
import os
import shutil

import numpy as np
import pytest

import cases
from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "plugins", "gauss_plugin.cu")
OUT = os.path.join(HERE, "plugins", "_build", "gauss_plugin.so")

# kinds of the test plugin
IDX_GAUSS, SUM_GAUSS, BLOCK_GAUSS = 0, 1, 2
SQNORM, POSITION, SHIFTED, LOGPDF_DEP, GRAD_DEP, SQUARE_DEP = 0, 1, 2, 3, 4, 5
GAUSS_ALL_MOVE, SINGLE_INDEX_MOVE, PAIR_MOVE, INDEPENDENCE_MOVE = 0, 1, 2, 3


@pytest.fixture(scope="module")
def plugin_path():
    if not shutil.which("nvcc") and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc is not available")
    from mcintegratorplusplus_gb300 import build
    return build.build_plugin(SRC, OUT)


def test_plugin_exports_and_loads(plugin_path):
    """The plugin's entry points answer without a GPU; the library accepts it and refuses a
    library that is not a plugin."""
    P = ctypes.CDLL(plugin_path)
    assert P.mcig_plugin_abi() == 1
    assert P.mcig_plugin_npdf() == 3 and P.mcig_plugin_nobs() == 6
    assert P.mcig_plugin_pdf_nproto(IDX_GAUSS, 5) == 5
    assert P.mcig_plugin_pdf_nproto(IDX_GAUSS, 65) == -1  # above max_nproto
    assert P.mcig_plugin_pdf_nproto(SUM_GAUSS, 40) == 1
    assert P.mcig_plugin_obs_nvals(POSITION, 7) == 7 and P.mcig_plugin_obs_nvals(SQNORM, 7) == 1
    assert P.mcig_plugin_nmove() == 4
    nproto, nstep, rate = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    par = (ctypes.c_double * 1)(0.8)
    P.mcig_plugin_move_info.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    assert P.mcig_plugin_move_info(PAIR_MOVE, 6, None, 0, ctypes.byref(nproto), ctypes.byref(nstep), ctypes.byref(rate)) == 0
    assert (nproto.value, nstep.value, rate.value) == (0, 2, 2. / 6)
    assert P.mcig_plugin_move_info(INDEPENDENCE_MOVE, 6, par, 1, ctypes.byref(nproto), ctypes.byref(nstep),
                                   ctypes.byref(rate)) == 0
    assert (nproto.value, nstep.value) == (1, 0)
    assert P.mcig_plugin_move_info(4, 6, None, 0, ctypes.byref(nproto), ctypes.byref(nstep), ctypes.byref(rate)) == -1
    s0, idx = (ctypes.c_double * 2)(), (ctypes.c_int * 6)()
    P.mcig_plugin_move_steps.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_void_p]
    assert P.mcig_plugin_move_steps(PAIR_MOVE, 6, None, 0, 2, s0, idx) == 0
    assert list(s0) == [0.05, 0.1] and list(idx) == [0, 0, 0, 1, 1, 1]
    import mcintegratorplusplus_gb300 as mcig
    pl = mcig.Plugin(plugin_path)
    assert (pl.npdf, pl.nobs, pl.nmove) == (3, 6, 4)
    assert pl.pdf(2) == mcig.PDF_USER + 2 and pl.obs(1) == mcig.OBS_USER + 1
    from mcintegratorplusplus_gb300 import _lib
    with pytest.raises(ValueError, match="plugin"):
        mcig.Plugin(_lib.lib_path())


@pytest.fixture(scope="module")
def mcig():
    import mcintegratorplusplus_gb300 as m
    return m


@pytest.fixture(scope="module")
def plugin(mcig, plugin_path):
    return mcig.Plugin(plugin_path)


def _run(mcig, plugin, ndim, nchains, prec, move, pdfs, obs, ms=None, seed=77, nmc=4096, ndecorr=200):
    m = mcig.MCI(ndim, nchains, precision=prec)
    m.setPlugin(plugin)
    m.setSeed(seed)
    if move[0] == "user":  # ("user", k, params): the plugin's k-th trial move
        m.setUserMove(move[1], move[2])
    else:
        m.setTrialMove(*move)
    for kind, par in pdfs:
        m.addSamplingFunction(kind, par)
    if ms is not None:
        nsub, subpdfs = ms
        m.setMultiStepMove(nsub, mcig.SRRD_UNIFORM, 1, 0.6)
        for kind, par in subpdfs:
            m.addMultiStepSamplingFunction(kind, par)
    for kind, par, bs, nskip, est in obs:
        m.addObservable(kind, par, bs, nskip, bs > 0, est)
    m.setNdecorrelationSteps(ndecorr)
    avg, err = m.integrate(nmc)
    data = [m.getObsData(o) for o in range(len(obs))]
    return dict(avg=avg, err=err, acc=m.getAcceptanceRate(), data=data, steps=m.getMRT2Steps(),
                chains=m.getChainResults(), x=m.getX())


def _assert_same(a, b):
    np.testing.assert_array_equal(a["avg"], b["avg"])
    np.testing.assert_array_equal(a["err"], b["err"])
    np.testing.assert_array_equal(a["steps"], b["steps"])
    np.testing.assert_array_equal(a["x"], b["x"])
    assert a["acc"] == b["acc"]
    for u, v in zip(a["data"], b["data"]):
        np.testing.assert_array_equal(u, v)


@pytest.mark.gpu
def test_vec_move_updated_acceptance_equals_builtin_gauss(mcig, plugin):
    """One proto value per index with updatedAcceptance under single-coordinate moves (the
    partial path) against the built-in Gauss kind; Block and Full (nskip 2) accumulators."""
    move = (mcig.MOVE_VEC, mcig.SRRD_UNIFORM, 1)
    E = mcig.EST_UNCORRELATED, mcig.EST_CORRELATED
    u = _run(mcig, plugin, 5, 64, mcig.PREC_FP64, move, [(plugin.pdf(IDX_GAUSS), ())],
             [(plugin.obs(SQNORM), (), 16, 1, E[0]), (plugin.obs(POSITION), (), 1, 2, E[1])])
    b = _run(mcig, plugin, 5, 64, mcig.PREC_FP64, move, [(mcig.PDF_GAUSS, ())],
             [(mcig.OBS_X2SUM, (), 16, 1, E[0]), (mcig.OBS_XND, (), 1, 2, E[1])])
    _assert_same(u, b)
    assert 0.3 < u["acc"] < 0.7


@pytest.mark.gpu
@pytest.mark.parametrize("prec_name", ["fp64", "fp32"])
def test_dependent_observables(mcig, plugin, prec_name):
    """Observables that depend on the sampling functions and on earlier observables
    (DependentObservableInterface.hpp:24-53): the log density from the plugin pdf's proto
    values equals the built-in LOGPDF observable of the same walk (FP64, bit for bit), the
    data its observationCallback prepared (the gradient -2 x) equals -2 x of the walker, and
    the square of the step's first observable equals the square of x.x."""
    prec = mcig.PREC_FP64 if prec_name == "fp64" else mcig.PREC_FP32
    move = (mcig.MOVE_VEC, mcig.SRRD_UNIFORM, 1)
    E = mcig.EST_UNCORRELATED
    u = _run(mcig, plugin, 5, 32, prec, move, [(plugin.pdf(IDX_GAUSS), ())],
             [(plugin.obs(SQNORM), (), 1, 1, E), (plugin.obs(LOGPDF_DEP), (), 1, 1, E),
              (plugin.obs(GRAD_DEP), (), 1, 1, E), (plugin.obs(SQUARE_DEP), (), 1, 1, E),
              (plugin.obs(POSITION), (), 1, 1, E)], nmc=1024)
    sq, lp, grad, sq2, pos = u["data"]
    np.testing.assert_array_equal(grad, -2 * pos)
    if prec == mcig.PREC_FP64:
        np.testing.assert_array_equal(sq2, sq * sq)
    else:  # the device squares the float value in float
        s32 = sq.astype(np.float32)
        np.testing.assert_array_equal(sq2, (s32 * s32).astype(np.float64))
    if prec == mcig.PREC_FP64:
        b = _run(mcig, plugin, 5, 32, prec, move, [(mcig.PDF_GAUSS, ())],
                 [(mcig.OBS_X2SUM, (), 1, 1, E), (mcig.OBS_LOGPDF, (), 1, 1, E)], nmc=1024)
        np.testing.assert_array_equal(sq, b["data"][0])
        np.testing.assert_array_equal(lp, b["data"][1])
    else:
        np.testing.assert_allclose(lp, -sq, rtol=1e-5)


@pytest.mark.gpu
def test_all_move_two_pdfs_with_parameters_equal_builtin(mcig, plugin):
    """A product of two user sampling functions, one with parameters, under all-moves; a user
    observable with a parameter against its built-in counterpart plus the shift."""
    move = (mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
    u = _run(mcig, plugin, 4, 128, mcig.PREC_FP64, move,
             [(plugin.pdf(SUM_GAUSS), ()), (plugin.pdf(BLOCK_GAUSS), (0, 2, 0.5))],
             [(plugin.obs(SQNORM), (), 32, 1, mcig.EST_MJBLOCKER), (plugin.obs(SHIFTED), (0.25,), 0, 1, mcig.EST_NOOP)])
    b = _run(mcig, plugin, 4, 128, mcig.PREC_FP64, move,
             [(mcig.PDF_GAUSS_SUM, ()), (mcig.PDF_GAUSS_BLOCK, (0, 2, 1.0))],  # 0.5 / 1.0^2 = 0.5
             [(mcig.OBS_X2SUM, (), 32, 1, mcig.EST_MJBLOCKER), (mcig.OBS_XND, (), 0, 1, mcig.EST_NOOP)])
    np.testing.assert_array_equal(u["avg"][:1], b["avg"][:1])
    np.testing.assert_array_equal(u["err"][:1], b["err"][:1])
    np.testing.assert_array_equal(u["steps"], b["steps"])
    np.testing.assert_array_equal(u["x"], b["x"])
    np.testing.assert_allclose(u["avg"][1:], b["avg"][1:] + 0.25, rtol=0, atol=1e-12)


@pytest.mark.gpu
def test_multistep_move_with_user_sub_pdfs_equals_builtin(mcig, plugin):
    """MultiStepMove whose sub-chain runs on user sampling functions (protos kept across the
    sub-steps, newToOld / oldToNew) inside a chain on a user sampling function."""
    move = (mcig.MOVE_ALL, mcig.SRRD_UNIFORM)
    obs = [(mcig.OBS_X2SUM, (), 16, 1, mcig.EST_UNCORRELATED)]
    u = _run(mcig, plugin, 5, 64, mcig.PREC_FP64, move, [(plugin.pdf(IDX_GAUSS), ())], obs,
             ms=(4, [(plugin.pdf(BLOCK_GAUSS), (0, 2, 0.5)), (plugin.pdf(BLOCK_GAUSS), (2, 5, 0.5))]), nmc=2048)
    b = _run(mcig, plugin, 5, 64, mcig.PREC_FP64, move, [(mcig.PDF_GAUSS, ())], obs,
             ms=(4, [(mcig.PDF_GAUSS_BLOCK, (0, 2, 1.0)), (mcig.PDF_GAUSS_BLOCK, (2, 5, 1.0))]), nmc=2048)
    _assert_same(u, b)


@pytest.mark.gpu
def test_replay_with_user_functors_reproduces_oracle(mcig, plugin):
    """Replaying the oracle's recorded draws, the user Gauss and observable reproduce the
    oracle's run of the reference's Gauss and X2Sum."""
    seeds = [3, 5]
    m = orc.OracleMCI(3, len(seeds))
    m.set_seeds(seeds)
    m.set_trial_move(cases.MOVE_VEC, cases.SRRD_UNIFORM, 1)
    m.add_sampling_function(cases.PDF_GAUSS)
    m.add_observable(cases.OBS_X2SUM, (), 8, 1, True, cases.EST_UNCORRELATED)
    m.set_ndecorrelation_steps(100)
    m.set_record(True)
    m.integrate(0, True, True)
    avg, err, ca, ce = m.integrate(4096, False, False, per_chain=True)
    tape, lens = m.get_tapes()
    g = mcig.MCI(3, len(seeds), precision=mcig.PREC_FP64)
    g.setPlugin(plugin)
    g.setTrialMove(mcig.MOVE_VEC, mcig.SRRD_UNIFORM, 1)
    g.addSamplingFunction(plugin.pdf(IDX_GAUSS))
    g.addObservable(plugin.obs(SQNORM), (), 8, 1, True, mcig.EST_UNCORRELATED)
    g.setNdecorrelationSteps(100)
    g.setReplay(tape, lens)
    g.integrate(0, True, True)
    gavg, gerr = g.integrate(4096, False, False)
    gca, gce = g.getChainResults()
    np.testing.assert_allclose(gca, ca, rtol=1e-12)
    np.testing.assert_allclose(gce, ce, rtol=1e-12)
    np.testing.assert_allclose(gavg, avg, rtol=1e-12)
    np.testing.assert_allclose(gerr, err, rtol=1e-12)
    a, _ = g.getCounts()
    oa, _ = m.counts()
    np.testing.assert_array_equal(a, oa)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["PREC_FP32", "PREC_FP32_ACC64"])
def test_float_paths_agree_with_builtin_and_analytic(mcig, plugin, prec):
    """Float walker: the log of the user acceptance ratio in the Metropolis test.  <sum x^2> of
    exp(-sum x^2) is ndim / 2."""
    p = getattr(mcig, prec)
    move = (mcig.MOVE_VEC, mcig.SRRD_UNIFORM, 2)
    ndim = 8
    u = _run(mcig, plugin, ndim, 2048, p, move, [(plugin.pdf(IDX_GAUSS), ())],
             [(plugin.obs(SQNORM), (), 32, 1, mcig.EST_UNCORRELATED)], nmc=4096, ndecorr=500)
    b = _run(mcig, plugin, ndim, 2048, p, move, [(mcig.PDF_GAUSS, ())],
             [(mcig.OBS_X2SUM, (), 32, 1, mcig.EST_UNCORRELATED)], nmc=4096, ndecorr=500, seed=78)
    for r in (u, b):
        assert abs(r["avg"][0] - ndim / 2) < 5 * r["err"][0], (r["avg"], r["err"])
    assert abs(u["avg"][0] - b["avg"][0]) < 5 * np.hypot(u["err"][0], b["err"][0])
    assert abs(u["acc"] - b["acc"]) < 0.01


@pytest.mark.gpu
def test_plugin_errors(mcig, plugin):
    m = mcig.MCI(3, 4, precision=mcig.PREC_FP64)
    with pytest.raises(ValueError, match="no plugin"):
        m.addSamplingFunction(mcig.PDF_USER)
    with pytest.raises(ValueError, match="no plugin"):
        m.addObservable(mcig.OBS_USER, (), 1, 1, False, mcig.EST_CORRELATED)
    m.setPlugin(plugin)
    with pytest.raises(ValueError, match="sampling functions"):
        m.addSamplingFunction(plugin.pdf(3))
    with pytest.raises(ValueError, match="observables"):
        m.addObservable(plugin.obs(7), (), 1, 1, False, mcig.EST_CORRELATED)
    m64 = mcig.MCI(64, 1)  # nproto(64) is at max_nproto: accepted
    m64.setPlugin(plugin)
    m64.addSamplingFunction(plugin.pdf(IDX_GAUSS))
    m.addSamplingFunction(plugin.pdf(IDX_GAUSS))
    m.addObservable(mcig.OBS_LOGPDF, (), 0, 1, False, mcig.EST_NOOP)
    with pytest.raises(NotImplementedError, match="LOGPDF"):
        m.integrate(64)
    m.popObservable()
    m.addObservable(plugin.obs(SQNORM), (), 0, 1, False, mcig.EST_NOOP)
    with pytest.raises(ValueError, match="plugin kinds"):
        m.setPlugin(None)
    m.setKernel(2)
    with pytest.raises(NotImplementedError):
        m.integrate(64)
    m.setKernel(0)
    m.integrate(64)
    f = mcig.MCI(4, 4, precision=mcig.PREC_FP32)
    f.setPlugin(plugin)
    f.addSamplingFunction(plugin.pdf(SUM_GAUSS))
    f.addObservable(mcig.OBS_X2SUM, (), 16, 1, True, mcig.EST_UNCORRELATED)
    f.setNdecorrelationSteps(10)
    with pytest.raises(NotImplementedError, match="batch"):
        mcig.Batch([f], 256)
    fl = mcig.Flow(4, nlayers=2)
    with pytest.raises(NotImplementedError, match="built-in"):
        mcig.integrate_flow(f, fl, 64)


# --- user trial moves (TrialMoveInterface as a device struct, MCIG_PLUGIN_MOVES)

@pytest.mark.gpu
@pytest.mark.parametrize("user_pdf", [False, True])
def test_user_gauss_all_move_equals_builtin_move(mcig, plugin, user_pdf):
    """The user Gaussian all-coordinate move draws the built-in move's normal deviates
    (UserRng::normal on the same Philox blocks) with the same arithmetic: FP64 runs with
    calibration, burn-in and sampling equal the built-in SRRDAllMove run bit for bit."""
    pdf = [(plugin.pdf(IDX_GAUSS), ())] if user_pdf else [(mcig.PDF_GAUSS, ())]
    obs = [(mcig.OBS_X2SUM, (), 16, 1, mcig.EST_UNCORRELATED), (mcig.OBS_XND, (), 0, 1, mcig.EST_NOOP)]
    u = _run(mcig, plugin, 5, 64, mcig.PREC_FP64, ("user", GAUSS_ALL_MOVE, ()), pdf, obs, nmc=2048)
    b = _run(mcig, plugin, 5, 64, mcig.PREC_FP64, (mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN), pdf, obs, nmc=2048)
    _assert_same(u, b)


def _oracle_tape(move, seeds, nmc=2048):
    m = orc.OracleMCI(4, len(seeds))
    m.set_seeds(seeds)
    m.set_trial_move(*move)
    m.add_sampling_function(cases.PDF_GAUSS)
    m.add_observable(cases.OBS_X2SUM, (), 8, 1, True, cases.EST_UNCORRELATED)
    m.add_observable(cases.OBS_XND, (), 0, 1, False, cases.EST_NOOP)
    m.set_ndecorrelation_steps(100)
    m.set_record(True)
    m.integrate(0, True, True)
    avg, err, ca, ce = m.integrate(nmc, False, False, per_chain=True)
    tape, lens = m.get_tapes()
    return dict(avg=avg, err=err, ca=ca, ce=ce, tape=tape, lens=lens, acc=m.counts()[0])


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["gauss_all", "single_index"])
def test_user_moves_replay_reproduce_oracle(mcig, plugin, which):
    """Replaying the oracle's recorded draws of the reference's SRRDAllMove (normal) and
    SRRDVecMove (uniform, vector length 1), the user moves that take the same draws in the
    same order (UserRng returns the recorded values) reproduce the oracle's run: calibration,
    burn-in, per-chain estimates and acceptance counts."""
    if which == "gauss_all":
        move, k = (cases.MOVE_ALL, cases.SRRD_GAUSSIAN, 0), GAUSS_ALL_MOVE
    else:
        move, k = (cases.MOVE_VEC, cases.SRRD_UNIFORM, 1), SINGLE_INDEX_MOVE
    seeds = [11, 12, 13]
    o = _oracle_tape(move, seeds)
    g = mcig.MCI(4, len(seeds), precision=mcig.PREC_FP64)
    g.setPlugin(plugin)
    g.setUserMove(k)
    g.addSamplingFunction(plugin.pdf(IDX_GAUSS))
    g.addObservable(plugin.obs(SQNORM), (), 8, 1, True, mcig.EST_UNCORRELATED)
    g.addObservable(plugin.obs(POSITION), (), 0, 1, False, mcig.EST_NOOP)
    g.setNdecorrelationSteps(100)
    g.setReplay(o["tape"], o["lens"])
    g.integrate(0, True, True)
    gavg, gerr = g.integrate(2048, False, False)
    gca, gce = g.getChainResults()
    np.testing.assert_allclose(gca, o["ca"], rtol=1e-12)
    np.testing.assert_allclose(gce, o["ce"], rtol=1e-12)
    np.testing.assert_allclose(gavg, o["avg"], rtol=1e-12)
    np.testing.assert_allclose(gerr, o["err"], rtol=1e-12)
    np.testing.assert_array_equal(g.getCounts()[0], o["acc"])


@pytest.mark.gpu
def test_noncontiguous_move_user_pdf_equals_builtin_pdf(mcig, plugin):
    """A move that changes two coordinates half the dimension apart: the user sampling
    function's updatedAcceptance walks the reported changed indices, the built-in one the
    indices between them (where the proposal equals the walker): the same FP64 run bit for
    bit, with two step sizes calibrated through the move's getStepSizeIndex."""
    obs = [(mcig.OBS_X2SUM, (), 16, 1, mcig.EST_UNCORRELATED)]
    u = _run(mcig, plugin, 6, 64, mcig.PREC_FP64, ("user", PAIR_MOVE, ()), [(plugin.pdf(IDX_GAUSS), ())], obs, nmc=2048)
    b = _run(mcig, plugin, 6, 64, mcig.PREC_FP64, ("user", PAIR_MOVE, ()), [(mcig.PDF_GAUSS, ())], obs, nmc=2048)
    _assert_same(u, b)
    assert u["steps"].shape == (64, 2)
    assert not np.array_equal(u["steps"][:, 0], u["steps"][:, 1])


@pytest.mark.gpu
@pytest.mark.parametrize("prec_name", ["fp64", "fp32"])
@pytest.mark.parametrize("k", [PAIR_MOVE, INDEPENDENCE_MOVE])
def test_user_moves_sample_the_target(mcig, plugin, prec_name, k):
    """<sum x^2> of exp(-sum x^2) is ndim / 2 under the two-coordinate move and under the
    independence move (move acceptance factor q(x)/q(x'), proto values kept across steps, no
    step sizes: findMRT2Step is skipped), standard error from the spread of the chain means."""
    prec = mcig.PREC_FP64 if prec_name == "fp64" else mcig.PREC_FP32
    ndim, nc = 6, 512
    params = (0.8,) if k == INDEPENDENCE_MOVE else ()
    r = _run(mcig, plugin, ndim, nc, prec, ("user", k, params), [(plugin.pdf(IDX_GAUSS), ())],
             [(mcig.OBS_X2SUM, (), 32, 1, mcig.EST_UNCORRELATED)], nmc=4096, ndecorr=500)
    ca = r["chains"][0][:, 0]
    z = abs(ca.mean() - ndim / 2) / (ca.std(ddof=1) / np.sqrt(nc))
    assert z < 4.0, (z, ca.mean())
    if k == INDEPENDENCE_MOVE:
        assert r["steps"].shape[1] == 0
        assert 0.3 < r["acc"] < 0.95, r["acc"]
    else:
        assert 0.35 < r["acc"] < 0.65, r["acc"]


@pytest.mark.gpu
def test_user_move_errors(mcig, plugin):
    m = mcig.MCI(4, 4, precision=mcig.PREC_FP64)
    with pytest.raises(ValueError, match="no plugin"):
        m.setUserMove(0)
    m.setPlugin(plugin)
    with pytest.raises(ValueError, match="trial moves"):
        m.setUserMove(4)
    m.setUserMove(GAUSS_ALL_MOVE)
    with pytest.raises(ValueError, match="plugin kinds"):
        m.setPlugin(None)
    m.addSamplingFunction(mcig.PDF_GAUSS)
    m.setKernel(2)
    with pytest.raises(NotImplementedError):
        m.integrate(64)
    m.setKernel(0)
    m.integrate(64)
    m.setTrialMove(mcig.MOVE_ALL)  # a built-in move again: the plugin may be detached
    m.setPlugin(None)
