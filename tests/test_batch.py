"""Batched integration of uneven integrals in one persistent launch (mcig_batch_*, CUDA graph).

* FP64 replay: batched integrals under the reference's recorded draws give the oracle's
  per-chain and combined results (the general double sampler in the batch).
* Block-separable sampler (the uneven-batch form: single-coordinate MultiStepMove on
  isotropic Gaussian factors over coordinate blocks, x.x per block) against the FP64
  oracle on the same Philox draws: a chain follows the oracle's walk unless a near-tie
  parts them, and then agrees to float rounding in its block means.
* Mixed batches: integrals of other forms run the general float sampler in the same launch
  and equal their own integrate with the general kernel bit for bit.
* Statistics: block moments against the analytic values (standard error from the chains'
  spread), the autotuner's choice (threads per block, unroll per ndim bucket) and a second
  graph replay that continues the chains.
"""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def blocks_of(rng, ndim):
    nb = int(min(ndim, rng.integers(2, 5)))
    cuts = np.sort(rng.choice(np.arange(1, ndim), nb - 1, replace=False)) if nb > 1 else np.array([], dtype=int)
    bounds = [0] + [int(c) for c in cuts] + [ndim]
    widths = 10.0 ** rng.uniform(np.log10(0.3), np.log10(3.0), nb)
    return bounds, widths


def configure(m, bounds, widths, nmc, nblocks=16, burnin=500, sub_srrd=0):
    """Product of isotropic Gaussian factors over the blocks, MultiStepMove with 4
    single-coordinate sub-moves on the same factors, x.x per block in a BlockAccumulator.

    With the sub-chain on the full target every outer step is accepted (MultiStepMove returns
    oldPDF/newPDF of its sub-pdf), so step calibration has nothing to measure (the reference
    doubles the step on every iteration): the sub-move step is set from the widths instead."""
    nb = len(widths)
    for k in range(nb):
        m.add_sampling_function(4, [bounds[k], bounds[k + 1], widths[k]])  # GAUSS_BLOCK
    m.set_multistep_move(4, sub_srrd, 1, float(2.0 * np.exp(np.mean(np.log(widths)))))
    for k in range(nb):
        m.multistep_add_pdf(4, [bounds[k], bounds[k + 1], widths[k]])
    m.set_nfind_mrt2_iterations(0)
    m.set_ndecorrelation_steps(burnin)
    m.add_observable(6, [nb] + bounds, nmc // nblocks, 1, False, 1)  # X2BLOCK, Block, Uncorrelated


def test_batch_fp64_replay_equals_oracle():
    import mcintegratorplusplus_gb300 as mcig
    rng = np.random.default_rng(11)
    specs = [(3, 2, 2048), (9, 3, 1024), (17, 2, 4096)]  # (ndim, chains, nmc)
    mcis, oracles = [], []
    for i, (ndim, nch, nmc) in enumerate(specs):
        bounds, widths = blocks_of(rng, ndim)
        o = orc.OracleMCI(ndim, nch)
        o.set_seeds(np.arange(nch, dtype=np.uint64) * np.uint64(101) + np.uint64(7 + i))
        configure(o, bounds, widths, nmc, burnin=200)
        o.set_record(True)
        oa, oe, oca, oce = o.integrate(nmc, True, True, per_chain=True)
        tape, lens = o.get_tapes()
        m = mcig.MCI(ndim, nch, precision=mcig.PREC_FP64)
        configure(m, bounds, widths, nmc, burnin=200)
        m.setReplay(tape, lens)
        mcis.append(m)
        oracles.append((oa, oe, oca, oce))
    b = mcig.Batch(mcis, [s[2] for s in specs])
    res = b.run()
    for m, (a, e), (oa, oe, oca, oce) in zip(mcis, res, oracles):
        ca, ce = m.getChainResults()
        np.testing.assert_allclose(ca, oca, rtol=1e-12)
        np.testing.assert_allclose(ce, oce, rtol=1e-12)
        np.testing.assert_allclose(a, oa, rtol=1e-12)
        np.testing.assert_allclose(e, oe, rtol=1e-12)


@pytest.mark.parametrize("sub_srrd", [0, 1])
def test_batch_block_separable_against_fp64_oracle_same_draws(sub_srrd):
    import mcintegratorplusplus_gb300 as mcig
    rng = np.random.default_rng(5)
    seed, nmc, nch = 4321, 4096, 24
    followed, total, worst = 0, 0, 0.0
    mcis, cases = [], []
    for ndim in (5, 12, 30, 64):
        bounds, widths = blocks_of(rng, ndim)
        m = mcig.MCI(ndim, nch, precision=mcig.PREC_FP32)
        m.setSeed(seed + ndim)
        configure(m, bounds, widths, nmc, sub_srrd=sub_srrd)
        mcis.append(m)
        cases.append((ndim, bounds, widths))
    b = mcig.Batch(mcis, [nmc] * len(mcis))
    b.run()
    for m, (ndim, bounds, widths) in zip(mcis, cases):
        ca, _ = m.getChainResults()
        o = orc.OracleMCI(ndim, nch)
        configure(o, bounds, widths, nmc, sub_srrd=sub_srrd)
        o.set_philox(seed + ndim, 0, None, layout=1)
        _, _, oca, _ = o.integrate(nmc, True, True, per_chain=True, nthreads=8)
        same = np.max(np.abs(m.getX() - o.get_x()), axis=1) < 1e-3
        assert np.array_equal(m.getStepCounters(), o.philox_counters())
        followed += int(same.sum())
        total += nch
        if same.any():
            rel = np.abs(ca[same] - oca[same]) / np.maximum(np.abs(oca[same]), 1.0)
            worst = max(worst, float(rel.max()))
    assert followed >= 0.8 * total, (followed, total)
    assert worst < 1e-4, worst
    print("\nblock-separable batch vs FP64 oracle (sub-move %s): %d/%d chains follow the whole run, block means "
          "max rel diff %.2e" % ("gaussian" if sub_srrd else "uniform", followed, total, worst))


def _gauss_handle(mcig, ndim, seed, nmc):
    g = mcig.MCI(ndim, 3, precision=mcig.PREC_FP32)
    g.setSeed(seed)
    g.addSamplingFunction(mcig.PDF_GAUSS)
    g.setTrialMove(mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
    g.setNdecorrelationSteps(100)
    g.addObservable(mcig.OBS_X2SUM, (), nmc // 16, 1, False, mcig.EST_UNCORRELATED)
    return g


def test_batch_mixed_forms_general_part_equals_solo():
    """Block-separable and other integrals in one launch: the others run the general float
    sampler and equal their own integrate with the general kernel bit for bit."""
    import mcintegratorplusplus_gb300 as mcig
    rng = np.random.default_rng(3)
    nmc = 2048
    mcis, solo = [], []
    for i, ndim in enumerate((4, 20, 40)):
        bounds, widths = blocks_of(rng, ndim)
        m = mcig.MCI(ndim, 3, precision=mcig.PREC_FP32)
        m.setSeed(70 + i)
        configure(m, bounds, widths, nmc)
        mcis += [m, _gauss_handle(mcig, ndim, 90 + i, nmc)]
        solo.append(_gauss_handle(mcig, ndim, 90 + i, nmc))
    b = mcig.Batch(mcis, [nmc] * len(mcis))
    res = b.run()
    for k, g2 in enumerate(solo):
        g2.setKernel(1)
        a, e = g2.integrate(nmc)
        avg, err = res[2 * k + 1]
        np.testing.assert_array_equal(a, avg)
        np.testing.assert_array_equal(e, err)


def test_batch_analytic_block_moments_and_autotune(tmp_path):
    import mcintegratorplusplus_gb300 as mcig
    rng = np.random.default_rng(7)
    mcis, exact, nmcs = [], [], []
    for i in range(48):
        ndim = int(rng.integers(1, 65))
        bounds, widths = blocks_of(rng, ndim)
        nmc = int(2 ** rng.integers(12, 15))
        m = mcig.MCI(ndim, 16, precision=mcig.PREC_FP32)
        m.setSeed(500 + i)
        configure(m, bounds, widths, nmc)
        mcis.append(m)
        exact.append(np.array([(bounds[k + 1] - bounds[k]) * widths[k] ** 2 for k in range(len(widths))]))
        nmcs.append(nmc)
    b = mcig.Batch(mcis, nmcs)
    block, unroll = b.autotune(str(tmp_path / "tune.txt"))
    assert block in (64, 128, 256) and all(u in (1, 2, 4) for u in unroll)
    assert mcig.Batch(mcis, nmcs).autotune(str(tmp_path / "tune.txt")) == (block, unroll)  # from the cache
    b.run()
    z = []
    for m, x in zip(mcis, exact):
        ca, _ = m.getChainResults()
        z.append(np.abs(ca.mean(0) - x) / (ca.std(0, ddof=1) / np.sqrt(ca.shape[0])))
    z = np.concatenate(z)
    assert np.mean(z < 3.0) > 0.97 and z.max() < 5.0, (np.mean(z < 3.0), z.max())
    # a second run continues the chains through the same graph
    res1 = b.run()
    res2 = b.run()
    assert not np.array_equal(res2[0][0], res1[0][0])
