"""The allocation-free MJBlocker entry point (mcig_mjblocker_estimate_noalloc).

It exists for callers that cannot call cudaMalloc (device memory owned by their
own pool, no device allocation allowed after start-up, or loops that must not
synchronize the device).  It takes device pointers and uses a static device
scratch array; its results must equal those of the allocating entry point
mcig_estimate on the same data, call after call.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as orc


def _lib():
    from mcintegratorplusplus_gb300 import _lib
    return _lib.load()


def test_noalloc_rejects_oversize_and_bad_n_without_device_work():
    L = _lib()
    one = ctypes.c_void_p(1)  # never dereferenced: the size checks come first
    max_values = 1 << 21
    assert L.mcig_mjblocker_estimate_noalloc(one, 1 << 20, 4, one, one, None) == 1
    assert b"exceeds the static scratch" in L.mcig_last_error()
    assert L.mcig_mjblocker_estimate_noalloc(one, 3000, 1, one, one, None) == 1
    assert b"power of two" in L.mcig_last_error()
    assert (1 << 19) * 4 == max_values  # largest accepted size for ndim 4


@pytest.mark.gpu
def test_noalloc_matches_allocating_estimator_call_after_call():
    import torch
    import mcintegratorplusplus_gb300 as mcig
    L = _lib()
    # calls in a row on different data: two small shapes, then the largest accepted sizes
    # (n * ndim == 2^21 values, the static scratch) with one coordinate and with four
    for seed, n, nd in ((1337, 1 << 15, 2), (7, 1 << 12, 17), (11, 1 << 21, 1), (13, 1 << 19, 4)):
        x = orc.splitmix64_ar1(seed, n, nd, 0.9 if nd <= 2 else 0.5)
        ref_avg, ref_err = mcig.estimate(mcig.EST_MJBLOCKER, x)  # allocating entry point
        dx = torch.from_numpy(x).cuda()
        davg = torch.full((nd,), float("nan"), dtype=torch.float64, device="cuda")
        derr = torch.full((nd,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = L.mcig_mjblocker_estimate_noalloc(ctypes.c_void_p(dx.data_ptr()), n, nd, ctypes.c_void_p(davg.data_ptr()),
                                               ctypes.c_void_p(derr.data_ptr()), None)
        assert rc == 0, L.mcig_last_error()
        torch.cuda.synchronize()
        np.testing.assert_allclose(davg.cpu().numpy(), ref_avg, rtol=1e-12, atol=0)
        np.testing.assert_allclose(derr.cpu().numpy(), ref_err, rtol=1e-12, atol=0)
