"""RayCaster pose state and helpers through the C ABI: pre/post multiplication of
every pose, the per-projection pose and camera getters, set_proj_cam_model, the
volume-centre and C-arm frames, and SimpleRayCasterWrapperFn (one projection
per camera of several objects, replace then accumulate, with intermediate
frames), each against the same computation done step by step."""
import numpy as np
import pytest

from tests.helpers import small_camera, small_volume
from xreg_gb300 import synth

pytestmark = pytest.mark.gpu


def _rc(xr, vols, cams, n):
    rc = xr.RayCasterLineIntCUDA()
    rc.set_volumes(vols)
    rc.set_camera_models(cams)
    rc.set_ray_step_size(0.5)
    rc.set_num_projs(n)
    rc.allocate_resources()
    return rc


def test_pre_post_multiply_and_getters(xr, oracle):
    vol = small_volume(41, (40, 36, 32), (1.5, 1.5, 1.5))
    cams = [small_camera((24, 28), 3.0), small_camera((24, 28), 2.5)]
    gt = synth.gt_pose(vol)
    poses = synth.sample_poses(vol, gt, 3, 5.0, 5.0, seed=2)
    rc = _rc(xr, [vol], cams, 6)
    rc.distribute_xforms_among_cam_models(poses)
    np.testing.assert_array_equal(rc.camera_model_proj_associations(), [0, 0, 0, 1, 1, 1])
    got = rc.xforms_cam_to_itk_phys()
    np.testing.assert_array_equal(got, np.concatenate([poses, poses]))
    pre = synth.perturb(vol, np.eye(4), [2.0, -1.0, 3.0], [4.0, 0.0, -2.0])
    post = synth.perturb(vol, np.eye(4), [-1.0, 0.5, 0.0], [0.0, 3.0, 1.0])
    rc.pre_multiply_all_xforms(pre)
    rc.post_multiply_all_xforms(post)
    x = rc.xforms_cam_to_itk_phys()
    # FrameTransform products in float, as xReg computes them (pre * pose, then * post)
    want = np.stack([oracle.frame_mul_f32(oracle.frame_mul_f32(pre, p), post) for p in poses])
    np.testing.assert_array_equal(x, np.concatenate([want] * 2))
    np.testing.assert_allclose(x, np.concatenate([pre @ poses @ post] * 2), rtol=0, atol=1e-4)
    rc.compute()
    mine = rc.projs()
    # the same poses given directly: identical images
    rc2 = _rc(xr, [vol], cams, 6)
    rc2.set_xforms_cam_to_itk_phys(x)
    rc2.set_camera_model_proj_associations(rc.camera_model_proj_associations())
    rc2.compute()
    np.testing.assert_array_equal(rc2.projs(), mine)
    # one projection's camera
    rc.set_proj_cam_model(0, 1)
    assert rc.camera_model_proj_associations()[0] == 1
    # poses given on the device are read back before multiplying
    import torch
    d = torch.from_numpy(poses.reshape(3, 16).copy()).cuda()
    rc.distribute_xforms_device(3, d.data_ptr())
    torch.cuda.synchronize()
    rc.pre_multiply_all_xforms(pre)
    np.testing.assert_array_equal(rc.xforms_cam_to_itk_phys()[:3],
                                  np.stack([oracle.frame_mul_f32(pre, p) for p in poses]))
    assert rc.num_vols() == 1 and rc.num_camera_models() == 2


def test_frames(xr):
    vol = small_volume(42, (41, 36, 30), (1.5, 1.2, 2.0))
    cam = small_camera((16, 16), 3.0)
    rc = _rc(xr, [vol], [cam], 1)
    np.testing.assert_allclose(rc.xform_img_center_to_itk_phys(0), vol.xform_img_center_to_itk_phys(),
                               rtol=0, atol=1e-12)
    c = rc.xform_cam_wrt_carm_center_of_rot(0)
    want = np.eye(4)
    want[2, 3] = -cam.focal_len / 2.0
    np.testing.assert_array_equal(c, want)


def test_simple_ray_caster_wrapper(xr):
    va = small_volume(43, (36, 32, 30), (1.5, 1.5, 1.5))
    vb = small_volume(44, (30, 30, 28), (1.2, 1.2, 1.2))
    cams = [small_camera((20, 24), 3.0), small_camera((20, 24), 2.0)]
    A = synth.perturb(va, synth.gt_pose(va), [3.0, 0.0, 1.0], [5.0, -2.0, 0.0])
    B = synth.perturb(vb, synth.gt_pose(vb), [-2.0, 1.0, 0.0], [-4.0, 3.0, 2.0])
    rc = _rc(xr, [va, vb], cams, 5)
    rc.set_num_projs(4)
    rc.distribute_xforms_among_cam_models(np.stack([A, B]))
    before = rc.camera_model_proj_associations().copy()
    projs = xr.simple_ray_cast(rc, [A, B])
    assert rc.num_projs() == 4
    np.testing.assert_array_equal(rc.camera_model_proj_associations(), before)
    # step by step: volume 0 replaces, volume 1 accumulates, one projection per camera
    ref = _rc(xr, [va, vb], cams, 2)
    ref.distribute_xforms_among_cam_models(A[None])
    ref.use_proj_store_replace_method()
    ref.compute(0)
    ref.distribute_xforms_among_cam_models(B[None])
    ref.use_proj_store_accum_method()
    ref.compute(1)
    for c in range(2):
        np.testing.assert_array_equal(projs[c], ref.proj(c))
    # intermediate frames about each volume, and a subset of volumes
    F = synth.perturb(va, np.eye(4), [0.0, 4.0, 0.0], [1.0, 0.0, 0.0])
    R = synth.perturb(va, np.eye(4), [1.0, 0.0, 0.0], [0.0, 0.0, 2.0])
    p2 = xr.simple_ray_cast(rc, [A], inter_frames=[F], inter_frames_wrt_vol=[True],
                            ref_frames_cam_world_to_vol=[R], vols_to_proj=[0])
    ref.distribute_xforms_among_cam_models((F @ A @ np.linalg.inv(F) @ R)[None])
    ref.use_proj_store_replace_method()
    ref.compute(0)
    for c in range(2):
        np.testing.assert_allclose(p2[c], ref.proj(c), rtol=1e-5, atol=1e-6)
