"""Job sets: several registrations' populations in one DRR launch.

Uneven jobs (volume sizes, voxel types, layouts, views, detectors, metrics,
population sizes) evaluated together must give exactly the values each gives
alone ("alone vs in the mix"), on any subset and order of jobs, through host and
device entry points."""
import numpy as np
import pytest

from tests.helpers import oracle_cams, oracle_geom, small_camera, small_volume
from xreg_gb300 import synth

pytestmark = pytest.mark.gpu


def _job(xr, seed, size, vt, det, nviews, kind, max_pop, cells=True):
    vol = small_volume(seed, size, (1.5, 1.5, 1.5))
    cams = [small_camera(det, 3.0)]
    if nviews > 1:
        from xreg_gb300.se3 import euler_xyz, rigid
        for k in range(1, nviews):
            R = euler_xyz(0.0, np.radians(15.0 + 10.0 * k), 0.0)
            c = np.array([0.0, 0.0, -synth.SOURCE_TO_CENTRE_MM])
            cam = small_camera(det, 3.0)
            cam.set_extrins(rigid(R, c - R @ c))
            cams.append(cam)
    rc = xr.RayCasterLineIntCUDA()
    rc.set_build_cell_layout(cells)
    rc.set_volume(vol, vt)
    rc.set_camera_models(cams)
    rc.set_ray_step_size(0.5)
    rng = np.random.default_rng(seed)
    ms = []
    for v in range(nviews):
        m = kind()
        m.set_fixed_image(rng.random(det).astype(np.float32))
        ms.append(m)
    obj = xr.PopulationObjective(rc, ms, max_pop)
    return obj, vol, cams, ms


def test_jobset_equals_alone(xr, oracle):
    jobs = [
        _job(xr, 1, (48, 44, 40), 0, (48, 52), 1, xr.ImgSimMetric2DGradNCCCUDA, 8),
        _job(xr, 2, (40, 36, 44), 1, (32, 36), 2, xr.ImgSimMetric2DNCCCUDA, 6),
        _job(xr, 3, (32, 32, 32), 2, (40, 40), 1, xr.ImgSimMetric2DPatchGradNCCCUDA, 4, cells=False),
        _job(xr, 4, (36, 40, 30), 0, (24, 28), 3, xr.ImgSimMetric2DGradNCCCUDA, 5, cells=False),
    ]
    pops = [7, 5, 3, 4]
    poses = [synth.sample_poses(j[1], synth.gt_pose(j[1]), p, 8.0, 10.0, seed=10 + i)
             for i, (j, p) in enumerate(zip(jobs, pops))]
    alone = [j[0].eval(p) for j, p in zip(jobs, poses)]
    js = xr.JobSet()
    mixed = js.eval([j[0] for j in jobs], poses)
    for a, m in zip(alone, mixed):
        np.testing.assert_array_equal(m, a)
    items, blocks = js.last_launch()
    assert 0 < blocks <= items  # one block per (tile, projection) item of the largest voxel-type group
    # subsets in another order, other population sizes
    sub = [jobs[2], jobs[0]]
    p2 = [poses[2][:2], poses[0][:5]]
    mixed2 = js.eval([j[0] for j in sub], p2)
    np.testing.assert_array_equal(mixed2[0], jobs[2][0].eval(p2[0]))
    np.testing.assert_array_equal(mixed2[1], jobs[0][0].eval(p2[1]))
    # job 0 against the oracle (FP32 DRR semantics + double grad-NCC)
    obj, vol, cams, ms = jobs[0]
    drr = oracle.drr_f32(vol.voxels, oracle_geom(vol), oracle_cams(cams), poses[0], step=0.5)
    fixed = np.random.default_rng(1).random((48, 52)).astype(np.float32)
    np.testing.assert_allclose(mixed[0], oracle.grad_ncc(fixed, drr), atol=1e-5, rtol=0)


def test_jobset_device_entry(xr):
    import torch
    jobs = [_job(xr, 5, (40, 40, 40), 0, (40, 44), 1, xr.ImgSimMetric2DGradNCCCUDA, 6),
            _job(xr, 6, (44, 40, 36), 1, (36, 40), 2, xr.ImgSimMetric2DGradNCCCUDA, 6)]
    poses = [synth.sample_poses(j[1], synth.gt_pose(j[1]), 6, 8.0, 10.0, seed=20 + i) for i, j in enumerate(jobs)]
    host = xr.JobSet().eval([j[0] for j in jobs], poses)
    js = xr.JobSet()
    s = torch.cuda.Stream()
    js.set_stream(s.cuda_stream)
    dx = [torch.from_numpy(p.reshape(-1, 16).copy()).cuda() for p in poses]
    ds = [torch.empty(6, dtype=torch.float32, device="cuda") for _ in jobs]
    torch.cuda.synchronize()
    js.eval_device([j[0] for j in jobs], [6, 6], [t.data_ptr() for t in dx], [t.data_ptr() for t in ds])
    s.synchronize()
    for h, d in zip(host, ds):
        np.testing.assert_array_equal(d.cpu().numpy(), h)


def test_jobset_errors(xr):
    from xreg_gb300 import _lib
    obj, vol, cams, ms = _job(xr, 7, (32, 32, 32), 0, (24, 24), 1, xr.ImgSimMetric2DGradNCCCUDA, 3)
    js = xr.JobSet()
    p = synth.sample_poses(vol, synth.gt_pose(vol), 4, 5.0, 5.0, seed=1)
    with pytest.raises(_lib.XRegError):
        js.eval([obj], [p])  # population above max_pop
    with pytest.raises(_lib.XRegError):
        js.eval([obj, obj], [p[:2], p[:2]])  # listed twice
    obj.close()
    with pytest.raises(_lib.XRegError):
        js.eval([obj], [p[:2]]) if obj._h else (_ for _ in ()).throw(_lib.XRegError(-1, "closed"))


def test_regi_step_errors_and_counts(xr):
    """xr_regi_jobset_step: refuses an unknown optimizer, a job without an
    objective or optimizer and an empty job list; reports lambda evaluations for
    a CMA-ES job and the ask size for a trust-region job."""
    from xreg_gb300 import _lib
    from xreg_gb300.cmaes import CMAES, TrustRegionDFO
    obj, vol, cams, ms = _job(xr, 8, (32, 32, 32), 0, (24, 24), 1, xr.ImgSimMetric2DGradNCCCUDA, 16)
    obj2, vol2, _, ms2 = _job(xr, 9, (32, 32, 32), 0, (24, 24), 1, xr.ImgSimMetric2DGradNCCCUDA, 16)
    js = xr.JobSet()
    C = vol.xform_img_center_to_itk_phys()
    start = synth.gt_pose(vol)
    es = CMAES(np.zeros(6), np.array([0.05] * 3 + [5.0] * 3), 6, seed=3)
    b = np.array([0.2] * 3 + [20.0] * 3)
    d = TrustRegionDFO(np.zeros(6), -b, b, 2.0, 0.01, 5)

    def job(o, opt, kind, bounds=None):
        j = _lib.xr_regi_step_job()
        j.obj = o._h.value if o is not None else None
        j.optimizer = kind
        j.opt = opt._h.value if opt is not None else None
        j.centre[:] = C.ravel().tolist()
        j.start_pose[:] = start.ravel().tolist()
        j.bounds[:] = (bounds if bounds is not None else np.zeros(6)).tolist()
        return j

    stop, ev = js.regi_step([job(obj, es, _lib.XR_REGI_CMAES, b), job(obj2, d, _lib.XR_REGI_DFO)])
    assert ev[0] == 6 and 1 <= ev[1] <= 14 and stop == [0, 0]
    for bad in (job(obj, es, 7), job(None, es, _lib.XR_REGI_CMAES), job(obj, None, _lib.XR_REGI_CMAES)):
        with pytest.raises(_lib.XRegError):
            js.regi_step([bad])
    with pytest.raises(_lib.XRegError):
        _lib.call("xr_regi_jobset_step", js._h, 0, None, None, None)


def test_pose_groups_are_identical(xr):
    """Job-set DRR items of 4 consecutive projections (xr_jobset_set_pose_groups):
    the same values and DRRs as the per-projection items, for tight populations
    (the 4 poses' rays within a voxel: one warp per 2x4-pixel sub-tile under all
    4 poses) and wide ones (one projection per pair of warps), populations that
    are not multiples of 4, several views, detectors not multiples of 8.  Mode 1
    groups the tight populations only; mode 2 every one."""
    jobs = [_job(xr, 31, (48, 44, 40), 0, (37, 45), 1, xr.ImgSimMetric2DGradNCCCUDA, 11),
            _job(xr, 32, (40, 36, 44), 1, (30, 34), 2, xr.ImgSimMetric2DGradNCCCUDA, 9),
            _job(xr, 33, (36, 40, 30), 2, (26, 29), 3, xr.ImgSimMetric2DGradNCCCUDA, 7)]
    for spread in ((10.0, 10.0), (0.02, 0.03)):
        poses = [synth.sample_poses(j[1], synth.gt_pose(j[1]), p, *spread, seed=40 + i)
                 for i, (j, p) in enumerate(zip(jobs, (11, 9, 6)))]
        js = xr.JobSet()
        base = js.eval([j[0] for j in jobs], poses)
        drr0 = [j[0].rc.projs().copy() for j in jobs]
        assert js.last_pose_grouped() == 0
        for mode in (2, 1):
            js.set_pose_groups(mode)
            for rep in range(2):
                got = js.eval([j[0] for j in jobs], poses)
                for a, b in zip(base, got):
                    np.testing.assert_array_equal(a, b)
                for j, d in zip(jobs, drr0):
                    np.testing.assert_array_equal(j[0].rc.projs(), d)
            # geometry, one DRR launch per voxel type (three here), one grad-NCC launch
            assert js.last_kernel_launches() == 1 + 3 + 1
            assert js.last_pose_grouped() == (3 if mode == 2 or spread[0] < 1.0 else 0), (mode, spread)
        with pytest.raises(xr.XRegError):
            js.set_pose_groups(3)
