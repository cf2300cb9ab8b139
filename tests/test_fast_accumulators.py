"""Accumulators of the register-resident float kernel against its own Full samples
(the reference's ut1 check that simple, block and full data agree,
test/ut1/main.cpp:341-345): on one trajectory, every Block mean is the mean of the
Full samples of its block and every Simple average the mean of all of them, for
one-value and vector observables, nskip 1 and 3, ndim at and below the padded width."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(mcig, ndim, nskip, prec, kernel):
    nc, nmc = 256, 960
    m = mcig.MCI(ndim, nc, precision=prec)
    m.setSeed(9)
    m.addSamplingFunction(mcig.PDF_GAUSS)
    m.setTrialMove(mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
    m.setNdecorrelationSteps(100)
    m.setKernel(kernel)
    naccu = 1 + (nmc - 1) // nskip
    bs = naccu // 8
    # x.x through all three accumulators, x_i through Full and Block (the value slots of
    # one integrate are limited to 2 MAXD + 8)
    m.addObservable(mcig.OBS_X2SUM, (), 1, nskip, False, mcig.EST_UNCORRELATED)   # Full (double here)
    m.addObservable(mcig.OBS_X2SUM, (), bs, nskip, False, mcig.EST_UNCORRELATED)  # Block
    m.addObservable(mcig.OBS_X2SUM, (), 0, nskip, False, mcig.EST_NOOP)           # Simple
    m.addObservable(mcig.OBS_XND, (), 1, nskip, False, mcig.EST_UNCORRELATED)
    m.addObservable(mcig.OBS_XND, (), bs, nskip, False, mcig.EST_UNCORRELATED)
    m.integrate(nmc, False, True)
    out = []
    for k, nv, has_simple in ((0, 1, True), (3, ndim, False)):
        full = m.getObsData(k).reshape(nc, naccu, nv)
        block = m.getObsData(k + 1).reshape(nc, 8, nv)
        simple = m.getObsData(k + 2).reshape(nc, nv) if has_simple else None
        out.append((full, block, simple, bs))
    return out


@pytest.mark.parametrize("ndim", [16, 13])
@pytest.mark.parametrize("nskip", [1, 3])
def test_fast_kernel_block_and_simple_equal_full_means(ndim, nskip):
    import mcintegratorplusplus_gb300 as mcig
    for full, block, simple, bs in run(mcig, ndim, nskip, mcig.PREC_FP32, 2):
        means = full.reshape(full.shape[0], -1, bs, full.shape[2]).mean(axis=2)
        # Kahan-compensated float sums against double sums of the same float samples
        np.testing.assert_allclose(block, means, rtol=2e-6, atol=2e-6)
        if simple is not None:
            np.testing.assert_allclose(simple, full.mean(axis=1), rtol=2e-6, atol=2e-6)


def test_fast_and_general_kernel_accumulate_alike():
    """The same float configuration through both kernels: identical Philox draws, so the
    trajectories agree up to float rounding of the log-density, and the accumulated data
    of the two kernels agree closely on the (vast) majority of chains."""
    import mcintegratorplusplus_gb300 as mcig
    a = run(mcig, 16, 1, mcig.PREC_FP32, 2)
    b = run(mcig, 16, 1, mcig.PREC_FP32, 1)
    for (fa, ba, sa, _), (fb, bb, sb, _) in zip(a, b):
        same = np.all(np.abs(fa - fb) < 1e-4 * (1 + np.abs(fb)), axis=(1, 2))
        assert same.mean() > 0.9, same.mean()
        np.testing.assert_allclose(ba[same], bb[same], rtol=1e-4, atol=1e-4)


@pytest.mark.parametrize("prec", ["PREC_FP32", "PREC_FP32_ACC64"])
def test_phase_fusion_equals_separate_launches(prec):
    """Calibration, burn-in and sampling of every chain in one launch give the results of the
    three launches: estimates, step sizes, walkers, counts and the accumulated data."""
    import mcintegratorplusplus_gb300 as mcig
    rng = np.random.default_rng(4)
    q, _ = np.linalg.qr(rng.normal(size=(16, 16)))
    P = q @ np.diag(10.0 ** rng.uniform(-1, 1, 16)) @ q.T

    def go(fuse):
        m = mcig.MCI(16, 2048, precision=getattr(mcig, prec))
        m.setSeed(21)
        m.setPhaseFusion(fuse)
        m.addSamplingFunction(mcig.PDF_GAUSS_PREC, P.ravel())
        m.setTrialMove(mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
        m.setNdecorrelationSteps(300)
        m.addObservable(mcig.OBS_X2SUM, (), 16, 1, True, mcig.EST_UNCORRELATED)
        m.addObservable(mcig.OBS_XND, (), 1, 1, False, mcig.EST_MJBLOCKER)
        avg, err = m.integrate(2048)
        ms = m.getLastTimings()
        return dict(avg=avg, err=err, steps=m.getMRT2Steps(), x=m.getX(), counts=m.getCounts(),
                    d0=m.getObsData(0), d1=m.getObsData(1), ms=ms)

    a, b = go(True), go(False)
    for k in ("avg", "err", "steps", "x", "d0", "d1"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    for u, v in zip(a["counts"], b["counts"]):
        np.testing.assert_array_equal(u, v)
    assert a["ms"]["launches"] < b["ms"]["launches"] and a["ms"]["calibration_ms"] < 0.05


@pytest.mark.parametrize("ndim,pdf,nfind", [(16, "PDF_GAUSS_PREC", -50), (13, "PDF_GAUSS_PREC", -50),
                                            (16, "PDF_GAUSS", -50), (16, "PDF_GAUSS_PREC", 7)])
def test_split_calibration_equals_one_lane(ndim, pdf, nfind):
    """The calibration whose tail runs on four lanes per chain gives every chain the step size,
    walker, Philox position and last-iteration counts of the one-lane calibration, bit for bit
    (a last warp with lanes beyond the chains, padded coordinates at ndim 13, a fixed number
    of iterations)."""
    import mcintegratorplusplus_gb300 as mcig
    rng = np.random.default_rng(11)
    q, _ = np.linalg.qr(rng.normal(size=(ndim, ndim)))
    P = q @ np.diag(10.0 ** rng.uniform(-1, 1, ndim)) @ q.T

    def go(split):
        m = mcig.MCI(ndim, 4091, precision=mcig.PREC_FP32)
        m.setSeed(5)
        m.setCalibrationSplit(split)
        if pdf == "PDF_GAUSS":
            m.addSamplingFunction(mcig.PDF_GAUSS)
        else:
            m.addSamplingFunction(mcig.PDF_GAUSS_PREC, P.ravel())
        m.setTrialMove(mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
        m.setNfindMRT2Iterations(nfind)
        m.integrate(0, True, False)
        return dict(steps=m.getMRT2Steps(), x=m.getX(), counts=m.getCounts())

    a, b = go(True), go(False)
    np.testing.assert_array_equal(a["steps"], b["steps"])
    np.testing.assert_array_equal(a["x"], b["x"])
    for u, v in zip(a["counts"], b["counts"]):
        np.testing.assert_array_equal(u, v)


def _uncorr_ref(full, nv):
    """MultiDimUncorrelatedEstimator (Estimators.cpp:125-155) per chain in double on the
    float Full samples [nchains][naccu * nv]"""
    x = full.reshape(full.shape[0], -1, nv).astype(np.float64)
    n = x.shape[1]
    avg = x.mean(axis=1)
    var = (x * x).sum(axis=1) / n - avg * avg
    err = np.where(var > 1e-300, np.sqrt(np.maximum(var, 0) / (n - 1.)), 0.)
    return avg, err, np.sqrt(np.maximum(var, 0))


@pytest.mark.parametrize("nskip", [1, 3])
def test_chunked_sampling_equals_one_launch(nskip):
    """Main sampling in chunks with the Full-sample estimator beside the next chunk
    (mcig_set_sampling_chunks) against one launch: identical accumulator data, chain
    estimates, averages, errors and counts; the Full estimates against the reference formula
    in double on the same float samples."""
    import mcintegratorplusplus_gb300 as mcig
    res = []
    for chunks in (1, 4, 3):  # 1: one launch (the default)
        nc, nmc = 512, 2400
        m = mcig.MCI(16, nc, precision=mcig.PREC_FP32)
        m.setSeed(21)
        m.setFullStorage(32)
        m.addSamplingFunction(mcig.PDF_GAUSS)
        m.setTrialMove(mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
        m.setNdecorrelationSteps(100)
        naccu = 1 + (nmc - 1) // nskip
        m.addObservable(mcig.OBS_X2SUM, (), naccu // 8, nskip, False, mcig.EST_UNCORRELATED)  # Block
        m.addObservable(mcig.OBS_XND, (), 1, nskip, False, mcig.EST_UNCORRELATED)              # Full
        m.addObservable(mcig.OBS_X2SUM, (), 1, 1, False, mcig.EST_UNCORRELATED)                # Full
        m.setSamplingChunks(chunks)
        avg, err = m.integrate(nmc)
        ca, ce = m.getChainResults()
        res.append([avg, err, ca, ce, *m.getCounts()] + [m.getObsData(o) for o in range(3)])
    nv_of = [1, 16, 1]
    for other in res[1:]:
        for a, b in zip(res[0], other):
            assert np.array_equal(a, b)
    for r in res:
        off = 1
        for o in (1, 2):
            avg, err, sd = _uncorr_ref(r[6 + o], nv_of[o])
            ca, ce = r[2][:, off:off + nv_of[o]], r[3][:, off:off + nv_of[o]]
            assert np.max(np.abs(ca - avg) / (np.abs(avg) + sd)) < 1e-6
            np.testing.assert_allclose(ce, err, rtol=2e-5)
            off += nv_of[o]


def _moments_run(mcig, prec, pdf, ndim, extra, second_xx=False):
    """Observables x.x and x_i in Block and float Full accumulators (the kernel variant that
    holds only those paths; at ndim 16 with one observable per group its straight-line layout);
    second_xx: one more x.x Full observable, every 2nd step (two in a group: the grouped
    loops); extra: one more observable (a constant, Simple) that makes the launch take the
    general observable code instead."""
    nc, nmc, nb = 300, 1200, 12
    m = mcig.MCI(ndim, nc, precision=prec)
    m.setSeed(21)
    m.setFullStorage(32)
    if pdf == "prec":
        rng = np.random.default_rng(3)
        q, _ = np.linalg.qr(rng.standard_normal((ndim, ndim)))
        m.addSamplingFunction(mcig.PDF_GAUSS_PREC, (q @ np.diag(10.0 ** rng.uniform(-1, 1, ndim)) @ q.T).ravel())
    else:
        m.addSamplingFunction(mcig.PDF_GAUSS)
    m.setTrialMove(mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
    m.setNdecorrelationSteps(200)
    m.setKernel(2)
    m.addObservable(mcig.OBS_X2SUM, (), nmc // nb, 1, False, mcig.EST_UNCORRELATED)
    m.addObservable(mcig.OBS_XND, (), nmc // nb, 1, False, mcig.EST_UNCORRELATED)
    m.addObservable(mcig.OBS_X2SUM, (), 1, 1, False, mcig.EST_UNCORRELATED)
    m.addObservable(mcig.OBS_XND, (), 1, 1, False, mcig.EST_UNCORRELATED)
    if second_xx:
        m.addObservable(mcig.OBS_X2SUM, (), 1, 2, False, mcig.EST_UNCORRELATED)
    if extra:
        m.addObservable(mcig.OBS_CONST, (2.5,), 0, 1, False, mcig.EST_NOOP)
    avg, err = m.integrate(nmc)
    ca, ce = m.getChainResults()
    nv = 2 + 2 * ndim + (1 if second_xx else 0)
    out = {"avg": avg[:nv], "err": err[:nv], "ca": ca[:, :nv], "ce": ce[:, :nv], "x": m.getX(),
           "steps": m.getMRT2Steps(), "ctr": m.getStepCounters(), "counts": np.stack(m.getCounts())}
    for o in range(5 if second_xx else 4):
        out["data%d" % o] = m.getObsData(o)
    return out


@pytest.mark.parametrize("prec_name,pdf,ndim,second_xx", [("PREC_FP32", "prec", 16, False),
                                                          ("PREC_FP32_ACC64", "prec", 16, False),
                                                          ("PREC_FP32", "prec", 16, True),
                                                          ("PREC_FP32", "gauss", 11, False)])
def test_moments_kernel_equals_general_observable_code(prec_name, pdf, ndim, second_xx):
    """The register-resident kernel holding only the x and x.x observable paths (straight-line
    for one observable per group, grouped loops otherwise) gives the general observable code's
    values bit for bit (same float products and sums)."""
    import mcintegratorplusplus_gb300 as mcig
    prec = getattr(mcig, prec_name)
    a = _moments_run(mcig, prec, pdf, ndim, False, second_xx)
    b = _moments_run(mcig, prec, pdf, ndim, True, second_xx)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
