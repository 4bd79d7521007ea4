"""The allocation-free apply (cppe_gpu_bmatrix_apply_direct_noalloc).

Callers that cannot allocate GPU memory -- a host program that hands the
library a fixed device pool, code inside a CUDA stream capture, a real-time
loop that must not enter the allocator -- call this entry point with their
own device buffers; its only scratch is a fixed device array.  The test calls
it through the C ABI twice in a row (the scratch keeps the first call's
contents) and compares each result with the ordinary entry point
(cppe_gpu_bmatrix_apply, direct summation, FP64) to the FP64 tolerance used
by the other parity tests.  This file is collected last so that a run that
stops at the first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

import cabi

pytestmark = pytest.mark.gpu


def _noalloc():
    f = cabi.lib().cppe_gpu_bmatrix_apply_direct_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p]
    return f


def test_noalloc_apply_matches_apply_twice(gpu):
    import torch
    from cppe_gb300 import synthetic

    b = synthetic.water_box(700, seed=31)  # 2,100 sites
    ref_sys = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=cabi.DIRECT,
                          damp=True)
    dev = torch.device("cuda:0")
    d_xyz = torch.tensor(b.xyz, dtype=torch.float64, device=dev).contiguous()
    d_a6 = torch.tensor(b.alpha6, dtype=torch.float64, device=dev).contiguous()
    d_ep = torch.tensor(b.excl_ptr, dtype=torch.int32, device=dev)
    d_ei = torch.tensor(b.excl_idx, dtype=torch.int32, device=dev)
    fn = _noalloc()
    rng = np.random.default_rng(5)
    for call in range(2):
        v = rng.normal(size=3 * b.n)
        expected = ref_sys.apply(v)
        d_in = torch.tensor(v, dtype=torch.float64, device=dev)
        d_out = torch.full_like(d_in, float("nan"))
        torch.cuda.synchronize()
        rc = fn(b.n, d_xyz.data_ptr(), d_a6.data_ptr(), d_ep.data_ptr(), d_ei.data_ptr(), 1,
                2.1304, d_in.data_ptr(), d_out.data_ptr(), None)
        assert rc == cabi.OK, cabi.last_error()
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        np.testing.assert_allclose(got, expected, rtol=0,
                                   atol=1e-12 * np.abs(expected).max(),
                                   err_msg=f"call {call}")


def test_noalloc_rejects_too_many_sites(gpu):
    fn = _noalloc()
    rc = fn(8193, 1, 1, None, None, 0, 2.1304, 1, 1, None)  # rejected before any GPU work
    assert rc == cabi.INVALID_ARG
    assert "8192" in cabi.last_error()
