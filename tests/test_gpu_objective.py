"""Population objective (poses -> DRRs -> per-view metric -> mean over views) on
the GPU against the oracle, plus the properties the batched path must keep at
full size: a pose's value is the same alone and inside a population, the
captured launch sequence replays bit-identically, and host and device entry
points agree."""
import numpy as np
import pytest

from tests.helpers import oracle_cams, oracle_geom, small_camera, small_volume
from xreg_gb300 import synth

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _objective(xr, vol, cams, fixed_imgs, kind, max_pop, step=0.5, stream=None):
    rc = xr.RayCasterLineIntCUDA()
    if stream is not None:
        rc.set_stream(stream)
    rc.set_volume(vol)
    rc.set_camera_models(cams)
    rc.set_ray_step_size(step)
    ms = []
    for f in fixed_imgs:
        m = kind()
        m.set_fixed_image(f)
        ms.append(m)
    return xr.PopulationObjective(rc, ms, max_pop), rc, ms


def _two_view_setup(seed=0):
    vol = small_volume(seed, (48, 44, 40), (1.5, 1.5, 1.5))
    from xreg_gb300.se3 import euler_xyz, rigid
    cams = [small_camera((48, 52), 3.0), small_camera((48, 52), 3.0)]
    R = euler_xyz(0.0, np.radians(25.0), 0.0)
    c = np.array([0.0, 0.0, -synth.SOURCE_TO_CENTRE_MM])
    cams[1].set_extrins(rigid(R, c - R @ c))
    return vol, cams


def _oracle_objective(oracle, vol, cams, fixed_imgs, poses, step, metric):
    n = len(poses)
    ci = np.repeat(np.arange(len(cams), dtype=np.int32), n)
    drr = oracle.drr_f32(vol.voxels, oracle_geom(vol), oracle_cams(cams), np.concatenate([poses] * len(cams)),
                         cam_idx=ci, step=step)
    vals = np.zeros(n)
    for v in range(len(cams)):
        vals += metric(fixed_imgs[v], drr[v * n:(v + 1) * n])
    return vals / len(cams)


@pytest.mark.parametrize("kind,metric", [("ImgSimMetric2DGradNCCCUDA", "grad_ncc"), ("ImgSimMetric2DNCCCUDA", "ncc"),
                                         ("ImgSimMetric2DPatchGradNCCCUDA", "patch_grad_ncc")])
def test_two_view_objective_matches_oracle(xr, oracle, kind, metric):
    vol, cams = _two_view_setup(1)
    gt = synth.gt_pose(vol)
    ci = np.arange(2, dtype=np.int32)
    fixed = oracle.drr_f32(vol.voxels, oracle_geom(vol), oracle_cams(cams), np.stack([gt, gt]), cam_idx=ci, step=0.5)
    fixed = [synth.add_noise(fixed[v], 0.01, 20 + v) for v in range(2)]
    obj, rc, ms = _objective(xr, vol, cams, fixed, getattr(xr, kind), 16)
    poses = synth.sample_poses(vol, gt, 9, 10.0, 20.0, seed=5)
    got = obj.eval(poses)
    ref = _oracle_objective(oracle, vol, cams, fixed, poses, 0.5, getattr(oracle, metric))
    np.testing.assert_allclose(got, ref, atol=TOL, rtol=0)
    # replays of the captured sequence are bit-identical
    np.testing.assert_array_equal(obj.eval(poses), got)
    np.testing.assert_array_equal(obj.eval(poses), got)


def test_alone_equals_in_the_mix_and_graph_path(xr, oracle):
    import torch
    vol, cams = _two_view_setup(2)
    gt = synth.gt_pose(vol)
    fixed = [np.random.default_rng(v).random((48, 52)).astype(np.float32) for v in range(2)]
    s = torch.cuda.Stream()
    obj, rc, ms = _objective(xr, vol, cams, fixed, xr.ImgSimMetric2DGradNCCCUDA, 32, stream=s.cuda_stream)
    poses = synth.sample_poses(vol, gt, 32, 10.0, 20.0, seed=7)
    mix = obj.eval(poses)
    alone = np.array([obj.eval(poses[i:i + 1])[0] for i in range(0, 32, 5)])
    np.testing.assert_array_equal(alone, mix[0:32:5])
    perm = np.random.default_rng(0).permutation(32)
    np.testing.assert_array_equal(obj.eval(poses[perm]), mix[perm])
    # device entry point (captured graph on a non-default stream) agrees with the host one
    d_x = torch.from_numpy(poses.reshape(32, 16).copy()).cuda()
    d_s = torch.empty(32, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for _ in range(3):
        with torch.cuda.stream(s):
            obj.eval_device(32, d_x.data_ptr(), d_s.data_ptr())
        s.synchronize()
        np.testing.assert_array_equal(d_s.cpu().numpy(), mix)


def test_population_errors(xr):
    from xreg_gb300 import _lib
    vol, cams = _two_view_setup(3)
    fixed = [np.zeros((48, 52), np.float32)] * 2
    obj, rc, ms = _objective(xr, vol, cams, fixed, xr.ImgSimMetric2DGradNCCCUDA, 4)
    with pytest.raises(_lib.XRegError):
        obj.eval(np.tile(np.eye(4), (5, 1, 1)))  # more than max_pop
    with pytest.raises(_lib.XRegError):
        obj.eval(np.full((1, 4, 4), np.inf))
    rc2 = xr.RayCasterLineIntCUDA()
    rc2.set_volume(vol)
    rc2.set_camera_models(cams[:1])
    with pytest.raises(_lib.XRegError):
        xr.PopulationObjective(rc2, ms, 4)  # two metrics, one camera


def test_destroy_in_any_order(xr):
    """Destroying a ray caster before the metric or objective bound to it must not
    crash; the dependent handles report an error instead."""
    from xreg_gb300 import _lib
    lib = _lib.load()
    vol, cams = _two_view_setup(4)
    fixed = [np.zeros((48, 52), np.float32)] * 2
    obj, rc, ms = _objective(xr, vol, cams, fixed, xr.ImgSimMetric2DGradNCCCUDA, 2)
    poses = np.tile(synth.gt_pose(vol), (2, 1, 1))
    obj.eval(poses)
    h_rc = rc.handle
    assert lib.xr_rc_destroy(h_rc) == 0
    rc._h = None  # already destroyed through the C ABI
    with pytest.raises(_lib.XRegError):
        obj.eval(poses)
    with pytest.raises(_lib.XRegError):
        ms[0].compute()
    obj.close()
    for m in ms:
        m.close()
