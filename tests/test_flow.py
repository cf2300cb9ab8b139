"""The learned proposal: affine-coupling flow kernels (bf16 tensor cores) against the
numpy oracle (oracle/flow_oracle.py), and the flow-assisted sampler against plain
Metropolis on a multimodal target."""
import numpy as np
import pytest

from oracle import flow_oracle as fo

D, L, H = 24, 8, 128


def random_params(seed, scale=0.02):
    rng = np.random.default_rng(seed)
    th = fo.init_params(D, L, H, seed).astype(np.float64)
    th += rng.standard_normal(th.shape) * scale
    return th.astype(np.float32)


def _to_bf16_bits(x):
    """float32 -> bf16 bit patterns, round to nearest even"""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((b + 0x7FFF + ((b >> 16) & 1)) >> 16).astype(np.uint16)


def _bf16_value(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.mark.gpu
@pytest.mark.parametrize("n,k", [(128, 16), (128, 128), (32, 128), (256, 64)])
def test_tcgen05_gemm_selftest(n, k):
    """The 5th-generation tensor-core path (tcgen05.mma, shared-memory descriptors of the
    no-swizzle K-major layout, f32 accumulator in tensor memory, tcgen05.ld) forms
    D = A B^T of bf16 operands as the float64 product of the same bf16 values does, to f32
    accumulation rounding."""
    import ctypes
    from mcintegratorplusplus_gb300 import _lib
    L = _lib.load()
    rng = np.random.default_rng(n * 1000 + k)
    a = _to_bf16_bits(rng.standard_normal((128, k)))
    b = _to_bf16_bits(rng.standard_normal((n, k)))
    d = np.full((128, n), np.nan, dtype=np.float32)
    rc = L.mcig_flow_tc_selftest(0, a.ctypes.data, b.ctypes.data, n, k,
                                 d.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    assert rc == 0, L.mcig_last_error()
    ref = _bf16_value(a) @ _bf16_value(b).T
    scale = np.sqrt(k)
    assert np.all(np.isfinite(d))
    assert np.max(np.abs(d - ref)) < 1e-5 * scale * 8, np.max(np.abs(d - ref))


def test_oracle_round_trip_and_gradient_by_finite_differences():
    perms = fo.permutations(D, 4, 7)
    rng = np.random.default_rng(0)
    th = fo.init_params(D, 4, 32, 1).astype(np.float64) + rng.standard_normal(fo.nparams(D, 4, 32)) * 0.005
    x = rng.standard_normal((8, D)) * 2
    z, lq = fo.inverse(th, x, D, 4, 32, perms, bf16=False)
    x2, lq2 = fo.forward(th, z, D, 4, 32, perms, bf16=False)
    assert np.abs(x2 - x).max() < 1e-10 and np.abs(lq2 - lq).max() < 1e-10
    loss, g = fo.loss_and_grad(th, x, D, 4, 32, perms, bf16=False)
    for i in rng.choice(th.size, 30, replace=False):
        tp, tm = th.copy(), th.copy()
        tp[i] += 1e-5
        tm[i] -= 1e-5
        fd = (-fo.inverse(tp, x, D, 4, 32, perms, bf16=False)[1].mean()
              + fo.inverse(tm, x, D, 4, 32, perms, bf16=False)[1].mean()) / 2e-5
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, np.abs(g).max()), i


def test_permutations_are_permutations():
    for p in fo.permutations(24, 8, 3):
        assert sorted(p.tolist()) == list(range(24))


@pytest.fixture(scope="module")
def mcig():
    import mcintegratorplusplus_gb300 as m
    m._lib.load()
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("tc", [0, 1, 2])
def test_flow_passes_match_oracle(mcig, tc):
    """The three pass kernels (register-fused mma.sync; tcgen05 with TMEM accumulators;
    mma.sync with shared-memory activations) against the oracle."""
    f = mcig.Flow(D, L, H, seed=11)
    f.set_tensor_path(tc)
    th = random_params(5)
    f.set_params(th)
    perms = fo.permutations(D, L, 11)
    rng = np.random.default_rng(1)
    z = rng.standard_normal((300, D))  # not a multiple of the 112-row pass tile nor the 128-row backward tile
    x, lq = f.forward(z)
    xo, lqo = fo.forward(th.astype(np.float64), z, D, L, H, perms, bf16=True)
    assert np.abs(x - xo).max() < 2e-2 * max(1.0, np.abs(xo).max())
    assert np.abs(lq - lqo).max() < 5e-2
    zi, lqi = f.inverse(x)
    zo, lqio = fo.inverse(th.astype(np.float64), x, D, L, H, perms, bf16=True)
    assert np.abs(zi - zo).max() < 2e-2 * max(1.0, np.abs(zo).max())
    assert np.abs(lqi - lqio).max() < 5e-2
    # the two directions agree on the same points (same network evaluations)
    assert np.abs(zi - z).max() < 1e-2
    assert np.abs(lqi - lq).max() < 1e-2


@pytest.mark.gpu
@pytest.mark.parametrize("Dd,Ld,n", [(D, L, 300), (6, 3, 200), (32, 4, 1000)])
def test_flow_fused_pass_equals_shared_memory_pass(mcig, Dd, Ld, n):
    """The register-fused pass (activations in registers) and the shared-memory pass form the
    same bf16 products in the same order: outputs and log q equal bit for bit, both ways."""
    rng = np.random.default_rng(8)
    th = (fo.init_params(Dd, Ld, H, 5).astype(np.float64) + rng.standard_normal(fo.nparams(Dd, Ld, H)) * 0.05)
    z = rng.standard_normal((n, Dd))
    out = []
    for tc in (0, 2):
        f = mcig.Flow(Dd, Ld, H, seed=5)
        f.set_tensor_path(tc)
        f.set_params(th.astype(np.float32))
        x, lq = f.forward(z)
        zi, lqi = f.inverse(x)
        out.append((x, lq, zi, lqi))
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b), np.abs(a - b).max()


@pytest.mark.gpu
@pytest.mark.parametrize("tc", [0, 1, 2])
def test_flow_odd_half_dimension_matches_oracle(mcig, tc):
    """D = 6 (d = 3): layer parameter blocks that do not start on 16-byte boundaries."""
    Dd, Ld = 6, 3
    f = mcig.Flow(Dd, Ld, H, seed=3)
    f.set_tensor_path(tc)
    rng = np.random.default_rng(4)
    th = (fo.init_params(Dd, Ld, H, 3).astype(np.float64) + rng.standard_normal(fo.nparams(Dd, Ld, H)) * 0.02)
    f.set_params(th.astype(np.float32))
    perms = fo.permutations(Dd, Ld, 3)
    z = rng.standard_normal((200, Dd))
    x, lq = f.forward(z)
    xo, lqo = fo.forward(th.astype(np.float32).astype(np.float64), z, Dd, Ld, H, perms, bf16=True)
    assert np.abs(x - xo).max() < 2e-2 * max(1.0, np.abs(xo).max())
    assert np.abs(lq - lqo).max() < 5e-2
    loss, g = f.loss_grad(xo)
    lo, go = fo.loss_and_grad(th.astype(np.float32).astype(np.float64), xo, Dd, Ld, H, perms, bf16=True)
    assert abs(loss - lo) < 1e-3 * abs(lo) + 1e-3
    assert np.linalg.norm(g - go) / np.linalg.norm(go) < 2e-2


@pytest.mark.gpu
def test_flow_gradient_matches_oracle(mcig):
    f = mcig.Flow(D, L, H, seed=11)
    th = random_params(9)
    f.set_params(th)
    perms = fo.permutations(D, L, 11)
    x = np.random.default_rng(2).standard_normal((512, D)) * 1.5
    loss, g = f.loss_grad(x)
    lo, go = fo.loss_and_grad(th.astype(np.float64), x, D, L, H, perms, bf16=True)
    assert abs(loss - lo) < 1e-3 * abs(lo) + 1e-3
    rel = np.linalg.norm(g - go) / np.linalg.norm(go)
    assert rel < 2e-2, rel
    # per-block agreement (every weight and bias block of every layer carries gradient)
    sizes = [int(np.prod(s)) for _, s in fo.layout(D, L, H)]
    off = 0
    for (name, _), n in zip(fo.layout(D, L, H), sizes):
        a, b = g[off:off + n], go[off:off + n]
        if np.linalg.norm(b) > 1e-6:
            assert np.linalg.norm(a - b) / np.linalg.norm(b) < 5e-2, (name, off)
        off += n


def c5_target(seed=2024, ndim=D):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((ndim, 2)))
    u1, u2 = Q[:, 0], Q[:, 1]
    means = np.stack([3 * u1, -3 * u1, 3 * u2, -3 * u2])
    params = np.concatenate([[4.0], np.full(4, 0.25), means.ravel(), np.ones(4 * ndim)])
    var_x1 = 1.0 + (means[:, 0] ** 2).mean()
    return params, means, var_x1


@pytest.mark.gpu
def test_flow_training_learns_the_mixture(mcig):
    params, means, _ = c5_target()
    rng = np.random.default_rng(3)
    comp = rng.integers(0, 4, 8192)
    x = means[comp] + rng.standard_normal((8192, D))
    f = mcig.Flow(D, L, H, seed=4)
    l0 = f.loss_grad(x[:2048])[0]
    last = f.train(x, 400, 1024, 2e-3)
    assert last < l0 - 5.0
    # the trained flow's samples populate all four modes
    xs, _ = f.forward(rng.standard_normal((4096, D)))
    near = np.argmin(((xs[:, None, :] - means[None]) ** 2).sum(-1), axis=1)
    frac = np.bincount(near, minlength=4) / len(near)
    assert np.all(frac > 0.1), frac


def _run_c5(mcig, use_flow, nchains=2048, nmc=1 << 13):
    params, means, var_x1 = c5_target()
    m = mcig.MCI(D, nchains, precision=mcig.PREC_FP32)
    m.setSeed(77)
    rng = np.random.default_rng(5)
    m.setX(rng.standard_normal((nchains, D)) * 3.0)
    m.addSamplingFunction(mcig.PDF_GAUSS_MIX, params)
    m.setTrialMove(mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
    m.setNdecorrelationSteps(1000)
    m.setFullStorage(32)
    m.addObservable(mcig.OBS_XI, [0], 1, 1, False, mcig.EST_MJBLOCKER)
    if use_flow:
        f = mcig.Flow(D, L, H, seed=6)
        avg, err, acc = mcig.integrate_flow(m, f, nmc, period=5, refresh=2048, train_steps=400, batch=2048, lr=2e-3)
    else:
        avg, err = m.integrate(nmc)
        acc = None
    ca, _ = m.getChainResults()
    ess_between = var_x1 * nchains / np.var(ca[:, 0])  # effective samples seen in the spread of chain means
    return avg[0], err[0], acc, ess_between, var_x1


@pytest.mark.gpu
def test_learned_proposal_beats_plain_mh(mcig):
    a_f, e_f, acc, ess_f, var_x1 = _run_c5(mcig, True)
    a_p, e_p, _, ess_p, _ = _run_c5(mcig, False)
    print("flow: %.4f +- %.4f acc %.3f ESS %.0f | plain: %.4f +- %.4f ESS %.0f" % (a_f, e_f, acc, ess_f, a_p, e_p, ess_p))
    assert acc > 0.05
    assert abs(a_f) < 4.0 * max(e_f, np.sqrt(var_x1 / ess_f))  # analytic mean 0
    assert ess_f > 5.0 * ess_p


@pytest.mark.gpu
def test_flow_sampler_unbiased_on_asymmetric_statistics(mcig):
    """The flow-assisted sampler (both log q of the Metropolis-Hastings ratio from the same
    density pass) against statistics a symmetric bias would not hide: <x_i^2> of every
    coordinate (analytic 1 + mean_k m_ki^2) and the occupancy of each of the four modes
    (analytic 1/4), both within 3 standard errors from the spread of the chain means."""
    params, means, _ = c5_target()
    nchains, nmc, nsub = 2048, 1 << 13, 256
    m = mcig.MCI(D, nchains, precision=mcig.PREC_FP32)
    m.setSeed(91)
    rng = np.random.default_rng(8)
    m.setX(rng.standard_normal((nchains, D)) * 3.0)
    m.addSamplingFunction(mcig.PDF_GAUSS_MIX, params)
    m.setTrialMove(mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
    m.setNdecorrelationSteps(1000)
    m.setFullStorage(32)
    m.addObservable(mcig.OBS_X2, (), 1, 1, False, mcig.EST_UNCORRELATED)
    m.addObservable(mcig.OBS_XND, (), 1, 1, False, mcig.EST_UNCORRELATED)
    f = mcig.Flow(D, L, H, seed=6)
    _, _, acc = mcig.integrate_flow(m, f, nmc, period=5, refresh=2048, train_steps=400, batch=2048, lr=2e-3)
    assert acc > 0.3
    ca, _ = m.getChainResults()
    x2 = ca[:, :D]
    exact = 1.0 + (means ** 2).mean(axis=0)
    z = np.abs(x2.mean(0) - exact) / (x2.std(0, ddof=1) / np.sqrt(nchains))
    assert z.max() < 3.5, z  # 24 coordinates: the largest of 24 normal deviates
    occ = np.zeros((nsub, 4))  # [chain][mode]: fraction of the chain's samples nearest each mode
    for c0 in range(0, nsub, 32):
        xs = m.getObsDataChains(1, c0, 32).reshape(32, nmc, D)
        d2 = (xs ** 2).sum(-1)[:, :, None] - 2.0 * xs @ means.T + (means ** 2).sum(-1)[None, None]
        near = np.argmin(d2, axis=2)
        occ[c0:c0 + 32] = np.stack([(near == k).mean(axis=1) for k in range(4)], axis=1)
    zo = np.abs(occ.mean(0) - 0.25) / (occ.std(0, ddof=1) / np.sqrt(nsub))
    assert zo.max() < 3.0, (occ.mean(0), zo)
    print("\nflow sampler: <x_i^2> max z %.2f, mode occupancy %s (max z %.2f), flow acceptance %.3f"
          % (z.max(), np.round(occ.mean(0), 4), zo.max(), acc))
