"""Parity at the benchmark's own sizes, against the CPU oracle.

* Batched population workload (the benchmark's headline): 256^3 float32
  phantom at 1 mm, detector 1536^2 at 0.194 mm downsampled 4x to 384^2, step
  0.5 mm, grad-NCC, a population of 100 poses (rotations N(0, 10 deg),
  translations N(0, 20 mm)).  Six of the hundred poses are checked against the
  oracle's FP32 restatement of xReg's ray caster: DRR max relative error
  <= 1e-4 (float32 volume), <= 2e-3 (FP16 volume), background pixels exactly
  equal, total sample count equal; grad-NCC within 1e-5 of the oracle's double
  arithmetic (float32 volume; 1e-4 with the FP16 volume, whose DRRs differ by up
  to 2e-3).  BF16 volumes are held to 2^-8, outside the 2e-3 half-precision
  tolerance: an 8-bit significand rounds a single voxel by up to 3.9e-3.
* Uneven multi-job step: the largest job of the uneven workload (512x512x300,
  FP16 volume, two views 25 deg apart, 384^2) evaluated in a job set beside a
  small job; one pose's DRRs and grad-NCC against the oracle.
"""
import numpy as np
import pytest

from tests.helpers import drr_rel_err, oracle_cams, oracle_geom
from xreg_gb300 import synth

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

PICK = [0, 13, 31, 50, 77, 99]


@pytest.fixture(scope="module")
def headline(oracle):
    w = synth.batched_population(0, 100)
    cams, geom = oracle_cams(w.cams), oracle_geom(w.vol)
    fixed = synth.add_noise(oracle.drr_f32(w.vol.voxels, geom, cams, synth.fixed_pose(w)[None], step=w.step)[0],
                            0.01, 2)
    poses = synth.sample_poses(w.vol, w.gt, 100, 10.0, 20.0, seed=11)
    ref, ns = oracle.drr_f32(w.vol.voxels, geom, cams, poses[PICK], step=w.step, count=True)
    ref_ncc = oracle.grad_ncc(fixed, ref)
    return w, fixed, poses, ref, ns, ref_ncc


def _population(xr, w, fixed, poses, vt):
    rc = xr.RayCasterLineIntCUDA()
    rc.set_volume(w.vol, vt)
    rc.set_camera_models(w.cams)
    rc.set_ray_step_size(w.step)
    m = xr.ImgSimMetric2DGradNCCCUDA()
    m.set_fixed_image(fixed)
    obj = xr.PopulationObjective(rc, [m], len(poses))
    vals = obj.eval(poses)
    drr = rc.projs()
    # the same poses alone, with the samples counted
    rc1 = xr.RayCasterLineIntCUDA()
    rc1.set_volume(w.vol, vt)
    rc1.set_camera_models(w.cams)
    rc1.set_ray_step_size(w.step)
    rc1.set_num_projs(len(PICK))
    rc1.allocate_resources()
    rc1.distribute_xforms_among_cam_models(poses[PICK])
    rc1.set_count_samples(True)
    rc1.compute()
    return vals, drr, rc1.projs(), rc1.last_num_samples()


@pytest.mark.parametrize("vt,drr_tol,ncc_tol", [(0, 1e-4, 1e-5), (1, 2e-3, 1e-4), (2, 2.0 ** -8, 1e-4)])
def test_headline_population_against_oracle(xr, oracle, headline, vt, drr_tol, ncc_tol):
    w, fixed, poses, ref, ns, ref_ncc = headline
    assert (w.vol.size, w.cams[0].num_det_rows, len(poses)) == ((256, 256, 256), 384, 100)
    vals, drr, alone, samples = _population(xr, w, fixed, poses, vt)
    assert samples == int(ns.sum())
    np.testing.assert_array_equal(drr[PICK], alone)
    rel, zero = drr_rel_err(drr[PICK], ref)
    assert zero == 0.0 and rel <= drr_tol, (vt, rel)
    assert np.max(np.abs(vals[PICK] - ref_ncc)) <= ncc_tol, (vals[PICK], ref_ncc)
    # the metric alone, on the GPU's own DRRs
    assert np.max(np.abs(vals[PICK] - oracle.grad_ncc(fixed, drr[PICK]))) <= 1e-5
    print(f"headline vt={vt}: DRR max rel {rel:.3e}, grad-NCC max abs {np.max(np.abs(vals[PICK] - ref_ncc)):.3e}")


def test_largest_uneven_job_in_a_jobset(xr, oracle):
    spec = synth.JobSpec(seed=4242, size=(512, 512, 300), spacing=(300.0 / 512,) * 3, view_angles=[0.0, 25.0],
                         ds_first=0.25, pop=20)
    vol = synth.phantom_volume(spec.size, spec.spacing, spec.seed)
    cams = synth.view_cameras(spec.view_angles, spec.ds_first)
    assert cams[0].num_det_rows == 384
    ocams, geom = oracle_cams(cams), oracle_geom(vol)
    gt = synth.gt_pose(vol)
    fixed = [synth.add_noise(f, 0.01, 5 + v) for v, f in
             enumerate(oracle.drr_f32(vol.voxels, geom, ocams, np.stack([gt, gt]), cam_idx=[0, 1], step=0.5))]
    poses = synth.sample_poses(vol, gt, spec.pop, 5.0, 10.0, seed=6)

    rc = xr.RayCasterLineIntCUDA()
    rc.set_volume(vol, 1)
    rc.set_camera_models(cams)
    rc.set_ray_step_size(0.5)
    ms = []
    for f in fixed:
        m = xr.ImgSimMetric2DGradNCCCUDA()
        m.set_fixed_image(f)
        ms.append(m)
    big = xr.PopulationObjective(rc, ms, spec.pop)
    # a small second job in the same launch
    svol = synth.phantom_volume((192, 192, 192), (300.0 / 192,) * 3, 7)
    scam = synth.view_cameras([0.0], 0.125)
    src = xr.RayCasterLineIntCUDA()
    src.set_volume(svol, 1)
    src.set_camera_models(scam)
    src.set_ray_step_size(0.5)
    sm = xr.ImgSimMetric2DGradNCCCUDA()
    sm.set_fixed_image(np.random.default_rng(3).random((192, 192)).astype(np.float32))
    small = xr.PopulationObjective(src, [sm], 30)
    spose = synth.sample_poses(svol, synth.gt_pose(svol), 30, 5.0, 10.0, seed=8)

    vals = xr.JobSet().eval([small, big], [spose, poses])[1]
    drr = rc.projs()  # [view][pose] in xReg's view-major order
    k = 3
    ref = oracle.drr_f32(vol.voxels, geom, ocams, np.stack([poses[k], poses[k]]), cam_idx=[0, 1], step=0.5)
    got = np.stack([drr[0 * spec.pop + k], drr[1 * spec.pop + k]])
    rel, zero = drr_rel_err(got, ref)
    assert zero == 0.0 and rel <= 2e-3, rel
    want = 0.5 * (oracle.grad_ncc(fixed[0], ref[0:1])[0] + oracle.grad_ncc(fixed[1], ref[1:2])[0])
    assert abs(vals[k] - want) <= 1e-4, (vals[k], want)
    print(f"largest job: DRR max rel {rel:.3e}, objective {vals[k]:.6f} vs oracle {want:.6f}")
