"""Precision study (32-D mixture of 8 anisotropic Gaussians): float walker arithmetic
with Kahan-compensated float block sums against double block sums on the same
trajectories, and both against the analytic moments."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NDIM, NCOMP = 32, 8


def c4_target(seed=404):
    rng = np.random.default_rng(seed)
    means = rng.standard_normal((NCOMP, NDIM)) * 3.0
    widths = 10.0 ** rng.uniform(np.log10(0.3), np.log10(3.0), (NCOMP, NDIM))
    w = rng.dirichlet(np.ones(NCOMP))
    params = np.concatenate([[NCOMP], w, means.ravel(), widths.ravel()])
    m1 = (w[:, None] * means).sum(0)                          # E[x_i]
    m2 = (w[:, None] * (widths ** 2 + means ** 2)).sum(0)     # E[x_i^2]
    return params, w, means, widths, m1, m2


def exact_samples(n, w, means, widths, seed):
    rng = np.random.default_rng(seed)
    comp = rng.choice(len(w), n, p=w)
    return means[comp] + widths[comp] * rng.standard_normal((n, NDIM))


def run(mcig, prec, nchains, nmc, x0):
    params, *_ = c4_target()
    m = mcig.MCI(NDIM, nchains, precision=prec)
    m.setSeed(31)
    m.setX(x0)
    m.addSamplingFunction(mcig.PDF_GAUSS_MIX, params)
    m.setTrialMove(mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
    m.setNdecorrelationSteps(256)
    bs = nmc // 64
    m.addObservable(mcig.OBS_X2SUM, (), bs, 1, False, mcig.EST_UNCORRELATED)
    m.addObservable(mcig.OBS_XND, (), bs, 1, False, mcig.EST_UNCORRELATED)
    m.addObservable(mcig.OBS_X2, (), bs, 1, False, mcig.EST_UNCORRELATED)
    avg, err = m.integrate(nmc)
    data = np.concatenate([m.getObsData(o) for o in range(3)], axis=1)
    ca, _ = m.getChainResults()
    return avg, err, data, ca


def test_kahan_float_sums_match_double_sums_on_identical_trajectories():
    import mcintegratorplusplus_gb300 as mcig
    _, w, means, widths, m1, m2 = c4_target()
    nchains, nmc = 2048, 8192
    x0 = exact_samples(nchains, w, means, widths, 1)
    a_k, e_k, d_k, ca_k = run(mcig, mcig.PREC_FP32, nchains, nmc, x0)
    a_d, e_d, d_d, ca_d = run(mcig, mcig.PREC_FP32_ACC64, nchains, nmc, x0)
    # the walkers are identical (same float arithmetic and draws); only the sums differ
    rel = np.abs(d_k - d_d) / np.maximum(np.abs(d_d), 1e-3)
    assert rel.max() < 1e-5, rel.max()
    # analytic moments, with the error of the chain ensemble (chains start in exact samples)
    for avg, ca in ((a_k, ca_k), (a_d, ca_d)):
        sem = ca.std(0) / np.sqrt(nchains)
        exact = np.concatenate([[m2.sum()], m1, m2])
        z = np.abs(avg - exact) / sem
        assert np.all(z < 4.5), z.max()


def test_double_walker_agrees_with_analytic_moments():
    import mcintegratorplusplus_gb300 as mcig
    _, w, means, widths, m1, m2 = c4_target()
    nchains, nmc = 256, 2048
    x0 = exact_samples(nchains, w, means, widths, 2)
    avg, err, data, ca = run(mcig, mcig.PREC_FP64, nchains, nmc, x0)
    sem = ca.std(0) / np.sqrt(nchains)
    exact = np.concatenate([[m2.sum()], m1, m2])
    assert np.all(np.abs(avg - exact) / sem < 4.5)
