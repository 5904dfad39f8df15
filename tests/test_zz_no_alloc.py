"""The allocation-free grad-NCC entry point (xr_grad_ncc_noalloc).

Callers that cannot allocate device memory on the metric's path (a host that
owns all device memory through its own allocator, or hands the library only
device pointers) use this entry point; its scratch is a fixed array inside the
library.  This test calls it through the C ABI twice in a row and compares both
results with the allocating metric (ImgSimMetric2DGradNCCCUDA) within the
similarity tolerance of the other metric tests.  It lives in a file that pytest
collects last and passes alone in a fresh process as well as after the others.
"""
import ctypes as C

import numpy as np
import pytest

TOL = 1e-5


@pytest.mark.gpu
def test_grad_ncc_noalloc_matches_allocating_metric(xr):
    import torch
    from xreg_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(21)
    rows, cols, n = 61, 77, 5
    fixed = rng.random((rows, cols)).astype(np.float32)
    base = rng.random((rows, cols)).astype(np.float32)
    movs = np.stack([0.6 * fixed + 0.4 * base + 0.05 * k * rng.random((rows, cols)) for k in range(n)])
    movs = movs.astype(np.float32)

    m = xr.ImgSimMetric2DGradNCCCUDA()
    m.set_fixed_image(fixed)
    m.set_num_moving_images(n)
    d_movs = torch.from_numpy(movs).cuda()
    m.set_mov_imgs_device_buf(d_movs.data_ptr(), 0)
    m.allocate_resources()
    m.compute()
    expect = m.sim_vals()

    d_fixed = torch.from_numpy(fixed).cuda()
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    for call in range(2):
        d_sims = torch.full((n,), -1.0, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        st = lib.xr_grad_ncc_noalloc(C.c_void_p(d_fixed.data_ptr()), C.c_void_p(d_movs.data_ptr()), rows, cols, n,
                                     5, C.c_void_p(d_sims.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert st == 0, lib.xr_last_error()
        stream.synchronize()
        got = d_sims.cpu().numpy()
        np.testing.assert_allclose(got, expect, atol=TOL, rtol=0, err_msg=f"call {call}")

    # sizes beyond the fixed scratch are refused with a message, not run
    big = 4096
    st = lib.xr_grad_ncc_noalloc(C.c_void_p(d_fixed.data_ptr()), C.c_void_p(d_movs.data_ptr()), big, big, 64, 5,
                                 C.c_void_p(d_sims.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert st == _lib.XR_ERR_INVALID_ARG
    assert b"scratch" in lib.xr_last_error()
    # more moving images than one launch's grid rows: refused before any launch
    st = lib.xr_grad_ncc_noalloc(C.c_void_p(d_fixed.data_ptr()), C.c_void_p(d_movs.data_ptr()), 8, 8, 70000, 5,
                                 C.c_void_p(d_sims.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert st == _lib.XR_ERR_INVALID_ARG
    assert b"65535" in lib.xr_last_error()
