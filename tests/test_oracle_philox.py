"""The oracle's Philox draw source (orc_set_philox): the device kernels' counter layout.

A chain of the oracle that draws from the device streams must see, at its first step, the
move draws and the acceptance uniform that the float (layout 1) or double (layout 2)
kernels derive from Philox4x32-10 blocks (mcig_common.cuh move_draws / accept_draw):
checked here by recomputing one step by hand from orc_philox4x32_10 and comparing the
walker after an accepted step and the recorded acceptance margin.
"""
import math

import numpy as np

from oracle import oracle as orc

SEED = 0x123456789ABCDEF


def _block(step, chain, sub, seed=SEED):
    return orc.philox4x32_10([step & 0xFFFFFFFF, step >> 32, chain, sub], [seed & 0xFFFFFFFF, seed >> 32])


def _draws_float(step, chain, ndim, gauss):
    d = []
    for b in range((ndim + 3) // 4):
        q = _block(step, chain, b)
        if gauss:
            for w0, w1 in ((q[0], q[1]), (q[2], q[3])):
                u = ((w0 >> 8) + 0.5) * 2.0 ** -24
                r = math.sqrt(-2.0 * math.log(u))
                th = 2.0 * math.pi * ((w1 >> 8) * 2.0 ** -24 - 0.5)
                d += [r * math.cos(th), r * math.sin(th)]
        else:
            d += [(w >> 8) * 2.0 ** -24 * 2.0 - 1.0 for w in q]
    u = ((_block(step, chain, 1 << 12)[0] >> 8) + 1) * 2.0 ** -24
    return np.array(d[:ndim]), u


def _u01d(hi, lo):
    return float(((hi << 21) | (lo >> 11))) * 2.0 ** -53


def _draws_double(step, chain, ndim, gauss):
    d = []
    for b in range((ndim + 1) // 2):
        q = _block(step, chain, b)
        if gauss:
            u = 1.0 - _u01d(q[0], q[1])
            r = math.sqrt(-2.0 * math.log(u))
            a = 2.0 * math.pi * _u01d(q[2], q[3])
            d += [r * math.cos(a), r * math.sin(a)]
        else:
            d += [_u01d(q[0], q[1]) * 2.0 - 1.0, _u01d(q[2], q[3]) * 2.0 - 1.0]
    qa = _block(step, chain, 1 << 12)
    return np.array(d[:ndim]), _u01d(qa[0], qa[1])


def _one_step(layout, gauss, chain0=5, ctr0=17, ndim=5):
    o = orc.OracleMCI(ndim, 1)
    o.add_sampling_function(1)  # exp(-x.x)
    o.set_trial_move(0, 1 if gauss else 0, 0)
    o.set_mrt2step(0.3)
    x0 = np.linspace(-0.4, 0.5, ndim)
    o.set_x(x0)
    o.add_observable(0, (), 1, 1, False, 1)
    o.set_philox(SEED, chain0, [ctr0], layout=layout)
    o.set_record(True)
    o.integrate(2, False, False)
    d, u = (_draws_float if layout == 1 else _draws_double)(ctr0, chain0, ndim, gauss)
    xn = x0 + 0.3 * d
    a = math.exp(-(xn @ xn) + (x0 @ x0))
    bits, start = o.get_accept_bits(0)
    mg = o.get_margins(0)[start]
    assert abs(mg - (math.log(u) - math.log(a))) < 1e-12
    assert bits[start] == (u <= a)
    assert o.philox_counters()[0] == ctr0 + 2
    xs = o.obs_data(0)  # x.x after each step
    if bits[start]:
        assert abs(xs[0, 0] - xn @ xn) < 1e-12
    else:
        assert abs(xs[0, 0] - x0 @ x0) < 1e-12


def test_philox_float_layout_gaussian():
    _one_step(1, True)


def test_philox_float_layout_uniform():
    _one_step(1, False)


def test_philox_double_layout_gaussian():
    _one_step(2, True)


def test_philox_double_layout_uniform():
    _one_step(2, False)


def test_philox_counters_advance_one_per_step():
    o = orc.OracleMCI(3, 2)
    o.add_sampling_function(1)
    o.set_trial_move(0, 1, 0)
    o.set_nfind_mrt2_iterations(2)
    o.set_ndecorrelation_steps(10)
    o.add_observable(0, (), 1, 1, False, 1)
    o.set_philox(7, 0, [100, 0], layout=1)
    o.integrate(50, True, True)
    ms = int(max(100, math.sqrt(40000 * 3)))  # MIN_STAT
    assert list(o.philox_counters()) == [100 + 2 * ms + 10 + 50, 2 * ms + 10 + 50]
