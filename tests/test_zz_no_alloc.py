"""The allocation-free apply (cppe_gpu_bmatrix_apply_direct_noalloc).

Callers that cannot allocate GPU memory -- a host program that hands the
library a fixed device pool and forbids further cudaMalloc, a real-time loop
that must not enter the allocator -- call this entry point with their own
device buffers; its only scratch is a fixed device array.  The tests call it
through the C ABI twice in a row (the scratch keeps the first call's
contents) and compare each result with the ordinary entry point
(cppe_gpu_bmatrix_apply, direct summation, FP64) to the FP64 tolerance used
by the other parity tests, once at 2,100 sites on the default stream and once
at 8,190 sites (the scratch nearly full) on a side stream.  A warm call must
leave the device's free memory unchanged.  This file is collected last so
that a run that stops at the first failure has run every other test before it.
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


def _device_inputs(b, dev):
    import torch
    return (torch.tensor(b.xyz, dtype=torch.float64, device=dev).contiguous(),
            torch.tensor(b.alpha6, dtype=torch.float64, device=dev).contiguous(),
            torch.tensor(b.excl_ptr, dtype=torch.int32, device=dev),
            torch.tensor(b.excl_idx, dtype=torch.int32, device=dev))


def _check_twice(waters, seed, side_stream):
    import torch
    from cppe_gb300 import synthetic

    b = synthetic.water_box(waters, seed=seed)
    ref_sys = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=cabi.DIRECT,
                          damp=True)
    dev = torch.device("cuda:0")
    d_xyz, d_a6, d_ep, d_ei = _device_inputs(b, dev)
    fn = _noalloc()
    stream = torch.cuda.Stream() if side_stream else None
    handle = stream.cuda_stream if side_stream else None
    rng = np.random.default_rng(seed)
    for call in range(2):
        v = rng.normal(size=3 * b.n)
        expected = ref_sys.apply(v)
        d_in = torch.tensor(v, dtype=torch.float64, device=dev)
        d_out = torch.full_like(d_in, float("nan"))
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(0)[0]
        rc = fn(b.n, d_xyz.data_ptr(), d_a6.data_ptr(), d_ep.data_ptr(), d_ei.data_ptr(), 1,
                2.1304, d_in.data_ptr(), d_out.data_ptr(), handle)
        assert rc == cabi.OK, cabi.last_error()
        torch.cuda.synchronize()
        if call == 1:  # warm: the scratch address is known, nothing may be allocated
            assert torch.cuda.mem_get_info(0)[0] == free0, "device free memory changed"
        got = d_out.cpu().numpy()
        np.testing.assert_allclose(got, expected, rtol=0,
                                   atol=1e-12 * np.abs(expected).max(),
                                   err_msg=f"{b.n} sites, call {call}")
    ref_sys.close()


def test_noalloc_apply_matches_apply_twice(gpu):
    _check_twice(700, 31, side_stream=False)  # 2,100 sites, default stream


def test_noalloc_apply_near_the_limit_on_a_side_stream(gpu):
    _check_twice(2730, 32, side_stream=True)  # 8,190 sites: every source split in use


def test_noalloc_rejects_too_many_sites(gpu):
    fn = _noalloc()
    rc = fn(8193, 1, 1, None, None, 0, 2.1304, 1, 1, None)  # rejected before any GPU work
    assert rc == cabi.INVALID_ARG
    assert "8192" in cabi.last_error()


def test_noalloc_rejects_output_overlapping_input(gpu):
    import torch
    from cppe_gb300 import synthetic

    b = synthetic.water_box(20, seed=33)
    d_xyz, d_a6, d_ep, d_ei = _device_inputs(b, torch.device("cuda:0"))
    buf = torch.zeros(6 * b.n, dtype=torch.float64, device="cuda:0")
    fn = _noalloc()
    for out_ptr in (buf.data_ptr(), buf.data_ptr() + 8 * 3):  # same buffer, shifted by a site
        rc = fn(b.n, d_xyz.data_ptr(), d_a6.data_ptr(), d_ep.data_ptr(), d_ei.data_ptr(), 1,
                2.1304, buf.data_ptr(), out_ptr, None)
        assert rc == cabi.INVALID_ARG
        assert "overlaps" in cabi.last_error()


def test_noalloc_marks_coincident_sites(gpu):
    import torch
    from cppe_gb300 import synthetic

    b = synthetic.water_box(40, seed=34)
    xyz = b.xyz.copy()
    # site 7 (an H of molecule 2) onto site 30 (the O of molecule 10)
    xyz.reshape(-1, 3)[7] = xyz.reshape(-1, 3)[30]
    dev = torch.device("cuda:0")
    d_xyz = torch.tensor(xyz, dtype=torch.float64, device=dev)
    _, d_a6, d_ep, d_ei = _device_inputs(b, dev)
    d_in = torch.tensor(np.random.default_rng(3).normal(size=3 * b.n), device=dev)
    d_out = torch.zeros_like(d_in)
    rc = _noalloc()(b.n, d_xyz.data_ptr(), d_a6.data_ptr(), d_ep.data_ptr(), d_ei.data_ptr(),
                    1, 2.1304, d_in.data_ptr(), d_out.data_ptr(), None)
    assert rc == cabi.OK, cabi.last_error()
    got = d_out.cpu().numpy().reshape(-1, 3)
    bad = np.where(~np.isfinite(got).all(axis=1))[0]
    assert list(bad) == [7, 30]
