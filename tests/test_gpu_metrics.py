"""GPU similarity metrics against the CPU oracle (double arithmetic), through the
C ABI.  Tolerance: absolute difference of each similarity value <= 1e-5 (the NCC
tolerance of the workload definitions), for NCC, grad-NCC, patch NCC and patch
grad-NCC, with and without masks, smoothing variants, odd image sizes.
The moving images are the GPU ray caster's own DRRs, read in place."""
import numpy as np
import pytest

from tests.helpers import small_camera, small_volume
from xreg_gb300 import synth

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _drrs(xr, det=(64, 72), n=6, seed=0, px=2.5):
    vol = small_volume(seed, (48, 44, 40), (1.5, 1.5, 1.5))
    cam = small_camera(det, px)
    rc = xr.RayCasterLineIntCUDA()
    rc.set_volume(vol)
    rc.set_camera_model(cam)
    rc.set_ray_step_size(0.5)
    poses = synth.sample_poses(vol, synth.gt_pose(vol), n + 1, 8.0, 10.0, seed=seed + 3)
    rc.set_num_projs(n + 1)
    rc.allocate_resources()
    rc.distribute_xforms_among_cam_models(poses)
    rc.compute()
    imgs = rc.projs()
    fixed = synth.add_noise(imgs[0], 0.01, seed + 9)
    return rc, imgs, fixed


def _metric(xr, cls, rc, fixed, n, offset=1, **kw):
    m = cls()
    m.set_fixed_image(fixed)  # a mask needs the fixed image's size first
    for k, v in kw.items():
        getattr(m, k)(v)
    m.set_num_moving_images(n)
    m.set_mov_imgs_buf_from_ray_caster(rc, offset)
    m.allocate_resources()
    m.compute()
    return m.sim_vals()


def test_ncc(xr, oracle):
    rc, imgs, fixed = _drrs(xr)
    got = _metric(xr, xr.ImgSimMetric2DNCCCUDA, rc, fixed, 6)
    ref = oracle.ncc(fixed, imgs[1:])
    np.testing.assert_allclose(got, ref, atol=TOL, rtol=0)
    # identities on the GPU: self gives 1/(2n), negated-contrast gives 1 - 1/(2n)
    self_v = _metric(xr, xr.ImgSimMetric2DNCCCUDA, rc, imgs[0], 1, offset=0)
    assert abs(self_v[0] - 0.5 / imgs[0].size) < TOL


def test_ncc_masked(xr, oracle):
    rc, imgs, fixed = _drrs(xr, seed=1)
    mask = (np.random.default_rng(3).random(fixed.shape) > 0.4).astype(np.uint8)
    got = _metric(xr, xr.ImgSimMetric2DNCCCUDA, rc, fixed, 6, set_mask=mask)
    ref = oracle.ncc(fixed, imgs[1:], mask=mask)
    np.testing.assert_allclose(got, ref, atol=TOL, rtol=0)


@pytest.mark.parametrize("smooth", [5, 3, 0])
def test_grad_ncc(xr, oracle, smooth):
    rc, imgs, fixed = _drrs(xr, det=(70, 61), seed=2)
    got = _metric(xr, xr.ImgSimMetric2DGradNCCCUDA, rc, fixed, 6,
                  set_smooth_img_before_sobel_kernel_radius=smooth)
    ref = oracle.grad_ncc(fixed, imgs[1:], smooth_ksize=smooth)
    np.testing.assert_allclose(got, ref, atol=TOL, rtol=0)


def test_grad_ncc_masked(xr, oracle):
    rc, imgs, fixed = _drrs(xr, seed=4)
    mask = np.zeros(fixed.shape, np.uint8)
    mask[5:-7, 9:-3] = 1
    got = _metric(xr, xr.ImgSimMetric2DGradNCCCUDA, rc, fixed, 6, set_mask=mask)
    ref = oracle.grad_ncc(fixed, imgs[1:], smooth_ksize=5, mask=mask)
    np.testing.assert_allclose(got, ref, atol=TOL, rtol=0)


@pytest.mark.parametrize("radius,stride", [(5, 1), (3, 2), (4, 3)])
def test_patch_ncc(xr, oracle, radius, stride):
    rc, imgs, fixed = _drrs(xr, det=(45, 52), seed=5)
    got = _metric(xr, xr.ImgSimMetric2DPatchNCCCUDA, rc, fixed, 6, set_patch_radius=radius,
                  set_patch_stride=stride)
    ref = oracle.patch_ncc(fixed, imgs[1:], radius=radius, stride=stride)
    np.testing.assert_allclose(got, ref, atol=TOL, rtol=0)


@pytest.mark.parametrize("radius,stride,smooth", [(5, 1, 5), (3, 2, 3), (5, 1, 0)])
def test_patch_grad_ncc(xr, oracle, radius, stride, smooth):
    rc, imgs, fixed = _drrs(xr, det=(50, 47), seed=6)
    got = _metric(xr, xr.ImgSimMetric2DPatchGradNCCCUDA, rc, fixed, 6, set_patch_radius=radius,
                  set_patch_stride=stride, set_smooth_img_before_sobel_kernel_radius=smooth)
    ref = oracle.patch_grad_ncc(fixed, imgs[1:], smooth_ksize=smooth, radius=radius, stride=stride)
    np.testing.assert_allclose(got, ref, atol=TOL, rtol=0)


def test_device_buffer_input_and_offsets(xr, oracle):
    import torch
    rng = np.random.default_rng(11)
    imgs = rng.random((5, 33, 40)).astype(np.float32)
    fixed = rng.random((33, 40)).astype(np.float32)
    d = torch.from_numpy(imgs).cuda()
    m = xr.ImgSimMetric2DGradNCCCUDA()
    m.set_fixed_image(fixed)
    m.set_num_moving_images(3)
    m.set_mov_imgs_device_buf(d.data_ptr(), 2)
    m.allocate_resources()
    m.compute()
    np.testing.assert_allclose(m.sim_vals(), oracle.grad_ncc(fixed, imgs[2:]), atol=TOL, rtol=0)


def test_metric_errors(xr):
    from xreg_gb300 import _lib
    m = xr.ImgSimMetric2DPatchGradNCCCUDA()
    with pytest.raises(_lib.XRegError):
        m.allocate_resources()  # no fixed image
    m.set_fixed_image(np.zeros((20, 20), np.float32))
    m.set_mask(np.ones((20, 20), np.uint8))  # patch metrics take masks (weights, masked sums)
    with pytest.raises(_lib.XRegError):
        m.set_patch_options(use_fixed_img_patch_variances_as_wgts=1, use_mov_img_patch_variances_as_wgts=1)
    with pytest.raises(TypeError):
        m.set_patch_options(no_such_option=1)
    import ctypes
    o = _lib.xr_patch_options()
    _lib.call("xr_patch_options_default", ctypes.byref(o))
    plain = xr.ImgSimMetric2DNCCCUDA()
    with pytest.raises(_lib.XRegError):  # not a patch metric
        _lib.call("xr_sm_set_patch_options", plain.handle, ctypes.byref(o))
    with pytest.raises(_lib.XRegError):
        m.set_smooth_img_before_sobel_kernel_radius(7)
    with pytest.raises(_lib.XRegError):
        m.compute()


def test_host_buffer_input(xr, oracle):
    """set_mov_imgs_host_buf: host images copied to the device at each compute."""
    rc, imgs, fixed = _drrs(xr, seed=4)
    m = xr.ImgSimMetric2DGradNCCCUDA()
    m.set_fixed_image(fixed)
    m.set_num_moving_images(5)
    host = imgs[1:6].copy()
    m.set_mov_imgs_host_buf(host)
    m.allocate_resources()
    m.compute()
    np.testing.assert_allclose(m.sim_vals(), oracle.grad_ncc(fixed, host), atol=TOL, rtol=0)
    host[:] = imgs[2:7]  # the buffer is read again at every compute
    m.compute()
    np.testing.assert_allclose(m.sim_vals(), oracle.grad_ncc(fixed, imgs[2:7]), atol=TOL, rtol=0)


def test_metric_getters(xr):
    """fixed_image, mask, num_pix_per_proj and num_moving_images return what was set."""
    rng = np.random.default_rng(21)
    fixed = rng.random((33, 40)).astype(np.float32)
    mask = (rng.random((33, 40)) > 0.3).astype(np.uint8)
    m = xr.ImgSimMetric2DGradNCCCUDA()
    m.set_fixed_image(fixed)
    assert m.mask() is None
    m.set_mask(mask)
    m.set_num_moving_images(3)
    np.testing.assert_array_equal(m.fixed_image(), fixed)
    np.testing.assert_array_equal(m.mask(), mask)
    assert m.num_pix_per_proj() == 33 * 40 and m.num_moving_images() == 3
    m.set_mask(None)
    assert m.mask() is None
