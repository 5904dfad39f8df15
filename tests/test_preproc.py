"""Data preparation either side of the hot path: HU -> attenuation, the
fixed-image downsampling of a coarser registration level (DownsampleImage:
discrete Gaussian + cubic B-spline resampling) and ProjPreProc (boundary crop +
log remap), GPU against the oracle, and the oracle pinned by the identities its
algorithms guarantee (kernel sums, polynomial reproduction, log identities)."""
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
    # factor 1: no smoothing; the interpolating B-spline returns the samples
    rnd = np.random.default_rng(3).random((37, 41)).astype(np.float32)
    np.testing.assert_allclose(oracle.downsample_image(rnd, 1.0), rnd, rtol=1e-6, atol=1e-7)


def test_downsample_bspline_reproduces_quadratics(oracle):
    """A symmetric blur maps x^2 to x^2 + v (v = the truncated kernel's variance)
    and the cubic B-spline reproduces quadratics exactly away from the mirrored
    edges, so at factor 0.3 (non-integer sample positions c / 0.3) the interior
    equals (c / 0.3)^2 + v."""
    f = 0.3
    x = np.arange(200, dtype=np.float64)
    img = np.tile((x * x).astype(np.float32), (40, 1))
    taps = oracle.discrete_gaussian_taps((0.5 / f) ** 2)
    k = np.arange(len(taps))
    v = 2.0 * np.sum(k * k * taps)
    d = oracle.downsample_image(img, f)
    c = np.arange(d.shape[1])
    want = (c / f) ** 2 + v
    inner = slice(12, d.shape[1] - 12)
    np.testing.assert_allclose(d[5:-5, inner], np.tile(want[inner], (d.shape[0] - 10, 1)), rtol=2e-6)


def test_log_remap_oracle_identities(oracle):
    # constant image: I0 = the constant, every pixel maps to -log(1) = 0
    np.testing.assert_array_equal(oracle.log_remap(np.full((30, 20), 7.5, np.float32)), 0.0)
    # explicit I0: x = I0 e^-2 maps to 2
    img = np.full((8, 9), np.float32(np.e ** -2 * 3.0), np.float32)
    np.testing.assert_allclose(oracle.log_remap(img, use_max=False, i0=3.0), 2.0, rtol=1e-6)
    # non-positive pixels take -log(min_pos / I0)
    img = np.random.default_rng(4).uniform(0.5, 4.0, (25, 31)).astype(np.float32)
    img[3, 4] = 0.0
    img[10, 2] = -1.0
    out = oracle.log_remap(img, use_max=False, i0=4.0)
    mp = img[img > 1e-6].min()
    assert out[3, 4] == out[10, 2] == np.float32(-np.log(np.float32(mp / np.float32(4.0))))
    np.testing.assert_allclose(out[img > 0], -np.log(img[img > 0] / 4.0), rtol=1e-6, atol=1e-6)


def test_camera_crop_boundary(xr):
    cam = xr.CameraModel.naive(1020.0, 300, 280, 0.5, 0.5)
    cc = cam.crop_boundary(50)
    assert (cc.num_det_rows, cc.num_det_cols) == (200, 180)
    k0, k1 = np.array(cam.desc.intrins).reshape(3, 3), np.array(cc.desc.intrins).reshape(3, 3)
    np.testing.assert_array_equal(k1[:, :2], k0[:, :2])
    np.testing.assert_array_equal(k1[:2, 2], k0[:2, 2] - 50.0)
    assert cc.desc.focal_len == cam.desc.focal_len
    from xreg_gb300 import _lib
    with pytest.raises(_lib.XRegError):
        cam.crop_boundary(140)


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


@pytest.mark.gpu
@pytest.mark.parametrize("factor", [1.0, 0.5, 0.3])
def test_downsample_gpu_small_and_identity(xr, oracle, factor):
    from xreg_gb300 import api
    img = np.random.default_rng(9).random((15, 11)).astype(np.float32)  # lines shorter than the prefilter horizon
    got = api.downsample_image(img, factor)
    np.testing.assert_allclose(got, oracle.downsample_image(img, factor), rtol=1e-6, atol=1e-6)


@pytest.mark.gpu
def test_proj_preproc_gpu_matches_oracle(xr, oracle):
    from xreg_gb300 import api
    rng = np.random.default_rng(5)
    img = rng.uniform(100.0, 4000.0, (260, 300)).astype(np.float32)
    img[rng.random(img.shape) < 0.01] = 0.0  # dead pixels
    crop = api.crop_image_boundary(img, 50)
    np.testing.assert_array_equal(crop, img[50:-50, 50:-50])
    got = api.log_remap(crop)
    np.testing.assert_allclose(got, oracle.log_remap(crop), rtol=2e-6, atol=2e-6)
    got_i0 = api.log_remap(crop, use_max_as_i0=False, i0=5000.0)
    np.testing.assert_allclose(got_i0, oracle.log_remap(crop, use_max=False, i0=5000.0), rtol=2e-6, atol=2e-6)
    cam = xr.CameraModel.naive(1020.0, 260, 300, 0.5, 0.5)
    out, c = api.proj_preproc(img, cam)
    assert out.shape == (c.num_det_rows, c.num_det_cols) == (160, 200)
    np.testing.assert_allclose(out, oracle.log_remap(img[50:-50, 50:-50]), rtol=2e-6, atol=2e-6)
