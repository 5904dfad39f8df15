"""Data preparation either side of the hot path: HU -> attenuation and the
fixed-image downsampling of a coarser registration level (DownsampleImage:
discrete Gaussian + resampling), GPU against the oracle, and the oracle's
discrete Gaussian pinned by its defining identities."""
import numpy as np
import pytest


def test_discrete_gaussian_identities(oracle):
    for var in (0.25, 1.0, 4.0, 16.0):
        t = oracle.discrete_gaussian_taps(var)
        assert abs(t[0] + 2 * t[1:].sum() - 1.0) < 1e-12
        assert np.all(np.diff(t) < 0)  # decreasing away from the centre
        # the untruncated kernel has variance `var`; truncation at 1% mass keeps it close
        k = np.arange(len(t))
        v = 2 * np.sum(k * k * t)
        assert abs(v - var) < 0.2 * var
    # more smoothing -> wider kernel
    assert len(oracle.discrete_gaussian_taps(16.0)) > len(oracle.discrete_gaussian_taps(4.0))


def test_downsample_oracle_identities(oracle):
    img = np.full((64, 48), 3.25, np.float32)
    d = oracle.downsample_image(img, 0.25)
    assert d.shape == (16, 12)
    np.testing.assert_allclose(d, 3.25, rtol=1e-6)
    ramp = np.tile(np.arange(48, dtype=np.float32), (64, 1))
    d = oracle.downsample_image(ramp, 0.5)
    # a ramp is preserved by the symmetric blur away from the edges; output column c samples input 2c
    np.testing.assert_allclose(d[:, 4:-4], np.tile(2.0 * np.arange(4, 20), (32, 1)), atol=1e-4)


@pytest.mark.gpu
@pytest.mark.parametrize("factor", [0.5, 0.25, 0.125, 0.3])
def test_downsample_gpu_matches_oracle(xr, oracle, factor):
    from xreg_gb300 import api
    rng = np.random.default_rng(int(factor * 1000))
    img = rng.random((200, 152)).astype(np.float32) * 5.0
    got = api.downsample_image(img, factor)
    ref = oracle.downsample_image(img, factor)
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-6)


@pytest.mark.gpu
def test_hu_to_lin_att_gpu(xr, oracle):
    import torch
    from xreg_gb300 import api
    hu = np.random.default_rng(0).uniform(-1500, 2000, 100003).astype(np.float32)
    d_hu = torch.from_numpy(hu).cuda()
    d_mu = torch.empty_like(d_hu)
    torch.cuda.synchronize()
    api.hu_to_lin_att_device(d_hu.data_ptr(), hu.size, d_mu.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_mu.cpu().numpy(), oracle.hu_to_lin_att(hu))
