"""The fused evaluation path (one persistent kernel: DRR tiles, then each
image's grad-NCC computed tile by tile behind them) against the split path
(DRR launch, then the metric's launches) and the oracle.

Both paths run the same tile-moment and FP64-combine code on the same tiles,
so values and DRRs must be identical bit for bit; against the oracle the
usual tolerances hold (DRR <= 1e-4 float32 volume, grad-NCC <= 1e-5).  Image
sizes that are not multiples of the 16x16 DRR tiles or the 32x64 metric
tiles, masks, several views, populations below the objective's maximum, and
repeated steps (the kernel's counters reset themselves) are covered; a job
set of uneven jobs equals each job alone on both job-set steps (geometry, DRR
and one batched grad-NCC launch; geometry and one fused launch per voxel-type
group)."""
import numpy as np
import pytest

from tests.helpers import drr_rel_err, oracle_cams, oracle_geom, small_camera, small_volume
from xreg_gb300 import synth

pytestmark = pytest.mark.gpu


def _objective(xr, vol, cams, fixed, vt=0, max_pop=8, masks=None, kind=None):
    rc = xr.RayCasterLineIntCUDA()
    rc.set_volume(vol, vt)
    rc.set_camera_models(cams)
    rc.set_ray_step_size(0.5)
    ms = []
    for v, f in enumerate(fixed):
        m = (kind or xr.ImgSimMetric2DGradNCCCUDA)()
        m.set_fixed_image(f)
        if masks is not None:
            m.set_mask(masks[v])
        ms.append(m)
    return xr.PopulationObjective(rc, ms, max_pop), rc


def _views(nviews, det):
    cams = [small_camera(det, 3.0)]
    from xreg_gb300.se3 import euler_xyz, rigid
    for k in range(1, nviews):
        R = euler_xyz(0.0, np.radians(20.0 * k), 0.0)
        c = np.array([0.0, 0.0, -synth.SOURCE_TO_CENTRE_MM])
        cam = small_camera(det, 3.0)
        cam.set_extrins(rigid(R, c - R @ c))
        cams.append(cam)
    return cams


@pytest.mark.parametrize("det,nviews,vt,masked", [((48, 52), 1, 0, False), ((50, 70), 2, 0, True),
                                                  ((20, 24), 1, 1, False), ((97, 131), 3, 2, False),
                                                  ((64, 64), 2, 1, True)])
def test_fused_equals_split(xr, oracle, det, nviews, vt, masked):
    vol = small_volume(31, (44, 40, 36), (1.5, 1.5, 1.5))
    cams = _views(nviews, det)
    gt = synth.gt_pose(vol)
    rng = np.random.default_rng(5)
    fixed = [synth.add_noise(f, 0.01, 3 + v) for v, f in enumerate(
        oracle.drr_f32(vol.voxels, oracle_geom(vol), oracle_cams(cams), np.stack([gt] * nviews),
                       cam_idx=list(range(nviews)), step=0.5))]
    masks = [(rng.random(det) > 0.2).astype(np.uint8) for _ in range(nviews)] if masked else None
    obj, rc = _objective(xr, vol, cams, fixed, vt, 8, masks)
    for step, pop in enumerate((8, 5, 8)):  # repeated steps, a population below max_pop
        poses = synth.sample_poses(vol, gt, pop, 6.0, 8.0, seed=40 + step)
        obj.set_fused(True)
        fused = obj.eval(poses)
        drr_f = rc.projs()[:nviews * pop].copy()
        obj.set_fused(False)
        split = obj.eval(poses)
        drr_s = rc.projs()[:nviews * pop].copy()
        np.testing.assert_array_equal(drr_f, drr_s)
        # each path against the metric restated in double on the same DRRs
        mk = [None] * nviews if masks is None else masks
        want = np.mean([oracle.grad_ncc(fixed[v], drr_f[v * pop:(v + 1) * pop], mask=mk[v])
                        for v in range(nviews)], axis=0)
        np.testing.assert_allclose(split, want, atol=1e-5, rtol=0, err_msg="split path vs oracle")
        np.testing.assert_allclose(fused, want, atol=1e-5, rtol=0, err_msg="fused path vs oracle")
        np.testing.assert_array_equal(fused, split)
    if vt == 0 and not masked:
        ref = oracle.drr_f32(vol.voxels, oracle_geom(vol), oracle_cams(cams),
                             np.concatenate([poses] * nviews), cam_idx=np.repeat(np.arange(nviews), pop), step=0.5)
        rel, zero = drr_rel_err(drr_f, ref)
        assert zero == 0.0 and rel <= 1e-4
        want = np.mean([oracle.grad_ncc(fixed[v], ref[v * pop:(v + 1) * pop]) for v in range(nviews)], axis=0)
        np.testing.assert_allclose(fused, want, atol=1e-5, rtol=0)


def test_fused_device_entry_and_graph_path(xr):
    """eval_device on the fused path equals the split path's captured graph."""
    import torch
    vol = small_volume(32, (40, 40, 40), (1.5, 1.5, 1.5))
    cams = [small_camera((40, 44), 3.0)]
    fixed = [np.random.default_rng(2).random((40, 44)).astype(np.float32)]
    obj, _ = _objective(xr, vol, cams, fixed, 0, 6)
    poses = synth.sample_poses(vol, synth.gt_pose(vol), 6, 8.0, 10.0, seed=3)
    d = torch.from_numpy(poses.reshape(6, 16).copy()).cuda()
    out = {}
    for fused in (True, False):
        obj.set_fused(fused)
        ds = torch.empty(6, dtype=torch.float32, device="cuda")
        for _ in range(3):
            obj.eval_device(6, d.data_ptr(), ds.data_ptr())
        torch.cuda.synchronize()
        out[fused] = ds.cpu().numpy()
    np.testing.assert_array_equal(out[True], out[False])


def test_jobset_steps_launches_and_alone(xr):
    """Uneven jobs (sizes, views, detectors, voxel types, one NCC job that runs
    its own metric launches): values equal each job alone, on the batched split
    step (geometry, DRR per voxel group, one grad-NCC launch) and the fused step
    (geometry, one fused launch per voxel group)."""
    def job(seed, size, vt, det, nviews, kind=None):
        vol = small_volume(seed, size, (1.5, 1.5, 1.5))
        cams = _views(nviews, det)
        rng = np.random.default_rng(seed)
        fixed = [rng.random(det).astype(np.float32) for _ in range(nviews)]
        obj, _ = _objective(xr, vol, cams, fixed, vt, 7, None, kind)
        return obj, vol

    jobs = [job(1, (48, 44, 40), 1, (48, 52), 1), job(2, (40, 36, 44), 1, (32, 36), 2),
            job(3, (36, 40, 30), 1, (40, 40), 3)]
    poses = [synth.sample_poses(v, synth.gt_pose(v), 7 - i, 8.0, 10.0, seed=10 + i) for i, (_, v) in enumerate(jobs)]
    alone = [o.eval(p) for (o, _), p in zip(jobs, poses)]
    js = xr.JobSet()
    for fused, launches in ((False, 3), (True, 2)):
        js.set_fused(fused)
        for rep in range(2):
            mixed = js.eval([o for o, _ in jobs], poses)
            for a, m in zip(alone, mixed):
                np.testing.assert_array_equal(m, a)
            if rep:
                assert js.last_kernel_launches() == launches
    # mixed voxel types and an NCC job (moments, finalize and its mean over views after the DRR)
    more = jobs + [job(4, (40, 40, 40), 0, (36, 36), 1), job(5, (32, 36, 40), 2, (30, 34), 1),
                   job(6, (36, 36, 36), 0, (28, 28), 2, xr.ImgSimMetric2DNCCCUDA)]
    p2 = poses + [synth.sample_poses(v, synth.gt_pose(v), 5, 8.0, 10.0, seed=20 + i)
                  for i, (_, v) in enumerate(more[3:])]
    alone2 = [o.eval(p) for (o, _), p in zip(more, p2)]
    for fused, launches in ((False, 1 + 3 + 1 + 5), (True, 1 + 3 + 5)):
        js.set_fused(fused)
        for rep in range(2):
            mixed = js.eval([o for o, _ in more], p2)
            for a, m in zip(alone2, mixed):
                np.testing.assert_array_equal(m, a)
            if rep:
                assert js.last_kernel_launches() == launches
