"""Full-size workloads on the GPU.

* Precision workload: 512x512x400 phantom at 0.8x0.8x1 mm, detector 1536^2 at
  0.194 mm downsampled 2x to 768^2, one pose; float32, FP16 and BF16 volumes
  against the oracle's FP32 semantics (tolerances 1e-4 / 2e-3 / 2^-8 max relative)
  and patch grad-NCC (11x11, stride 1) against the oracle (1e-5).  Errors against
  the FP64 oracle are computed too (they include the float geometry of the
  reference algorithm itself) and must stay small over the body.
* Batched workload (256^3, 384^2, 100 poses): size-independent properties of the
  population path - a pose's value is identical alone and in the population,
  permuting the population permutes the values, FP16 stays within the metric
  tolerance of FP32.
"""
import json
import os

import numpy as np
import pytest

from tests.helpers import drr_rel_err, oracle_cams, oracle_geom
from xreg_gb300 import synth

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(scope="module")
def precision():
    w = synth.precision_large(0)
    return w, synth.fixed_pose(w)


def _drr(xr, w, pose, vt):
    rc = xr.RayCasterLineIntCUDA()
    rc.set_volume(w.vol, vt)
    rc.set_camera_models(w.cams)
    rc.set_ray_step_size(w.step)
    rc.set_num_projs(1)
    rc.allocate_resources()
    rc.distribute_xforms_among_cam_models(pose[None])
    rc.set_count_samples(True)
    rc.compute()
    out = rc.projs()
    return out, rc.last_num_samples()


def test_precision_workload_drr(xr, oracle, precision):
    w, pose = precision
    cams, geom = oracle_cams(w.cams), oracle_geom(w.vol)
    ref, ns = oracle.drr_f32(w.vol.voxels, geom, cams, pose[None], step=w.step, count=True)
    ref64 = oracle.drr_f64(w.vol.voxels, geom, cams, pose[None], step=w.step)
    assert w.cams[0].num_det_rows == 768
    assert int(ns.sum()) > 3e8  # ~0.47 G trilinear samples for this pose
    g32, s32 = _drr(xr, w, pose, 0)
    assert s32 == int(ns.sum())
    rel32, z32 = drr_rel_err(g32, ref)
    assert z32 == 0.0 and rel32 <= 1e-4, rel32
    g16, _ = _drr(xr, w, pose, 1)
    rel16, z16 = drr_rel_err(g16, ref)
    assert z16 == 0.0 and rel16 <= 2e-3, rel16
    gbf, _ = _drr(xr, w, pose, 2)
    relbf, zbf = drr_rel_err(gbf, ref)
    assert zbf == 0.0 and relbf <= 2.0 ** -8, relbf
    # against the FP64 oracle: the median relative error over the body is tiny
    body = ref64 > 0.1 * ref64.max()
    for g in (g32, g16):
        assert np.median(np.abs(g[body] - ref64[body]) / ref64[body]) < 1e-3
    report = {"workload": "512x512x400 @0.8x0.8x1 mm, 768^2, step %.2f mm, one pose" % w.step,
              "samples": int(ns.sum())}
    for name, g, rel in (("f32", g32, rel32), ("f16", g16, rel16), ("bf16", gbf, relbf)):
        r64 = np.abs(g[body] - ref64[body]) / ref64[body]
        report[name] = {"max_rel_vs_fp32_oracle": float(rel), "max_rel_vs_fp64_oracle_body": float(r64.max()),
                        "median_rel_vs_fp64_oracle_body": float(np.median(r64)),
                        "max_rel_vs_f32_volume_body": float(np.max(np.abs(g[body] - g32[body]) / g32[body]))}
    r = np.abs(ref[body] - ref64[body]) / ref64[body]
    report["fp32_oracle_itself"] = {"max_rel_vs_fp64_oracle_body": float(r.max()),
                                    "median_rel_vs_fp64_oracle_body": float(np.median(r))}
    _report("precision_drr", report)


def test_precision_workload_patch_grad_ncc(xr, oracle, precision):
    w, pose = precision
    cams, geom = oracle_cams(w.cams), oracle_geom(w.vol)
    fixed = synth.add_noise(oracle.drr_f32(w.vol.voxels, geom, cams, w.gt[None], step=w.step)[0], 0.01, 3)
    rc = xr.RayCasterLineIntCUDA()
    rc.set_volume(w.vol, 1)
    rc.set_camera_models(w.cams)
    rc.set_ray_step_size(w.step)
    m = xr.ImgSimMetric2DPatchGradNCCCUDA()
    m.set_fixed_image(fixed)
    obj = xr.PopulationObjective(rc, [m], 2)
    poses = np.stack([pose, w.gt])
    got = obj.eval(poses)
    drr = rc.projs()
    ref = oracle.patch_grad_ncc(fixed, drr, smooth_ksize=5, radius=5, stride=1)
    np.testing.assert_allclose(got, ref, atol=1e-5, rtol=0)
    assert got[1] < got[0]  # the ground-truth pose scores better
    _report("precision_patch_grad_ncc", {"gpu": got.tolist(), "oracle_fp64_on_same_drrs": ref.tolist(),
                                         "max_abs_diff": float(np.max(np.abs(got - ref)))})


def _report(name, d):
    """Prints an error summary; also writes it as JSON into XREG_GB300_REPORT_DIR when set."""
    print(name, json.dumps(d))
    out = os.environ.get("XREG_GB300_REPORT_DIR")
    if out:
        os.makedirs(out, exist_ok=True)
        with open(os.path.join(out, name + ".json"), "w") as f:
            json.dump(d, f, indent=1)


def test_batched_population_properties(xr):
    import torch
    w = synth.batched_population(0, 100)
    rc = xr.RayCasterLineIntCUDA()
    rc.set_volume(w.vol)
    rc.set_camera_models(w.cams)
    rc.set_ray_step_size(w.step)
    rc.set_num_projs(1)
    rc.allocate_resources()
    rc.distribute_xforms_among_cam_models(synth.fixed_pose(w)[None])
    rc.compute()
    fixed = synth.add_noise(rc.proj(0), 0.01, 2)
    rc.close()
    s = torch.cuda.Stream()
    vals = {}
    for vt in (0, 1):
        rcp = xr.RayCasterLineIntCUDA()
        rcp.set_stream(s.cuda_stream)
        rcp.set_volume(w.vol, vt)
        rcp.set_camera_models(w.cams)
        rcp.set_ray_step_size(w.step)
        m = xr.ImgSimMetric2DGradNCCCUDA()
        m.set_fixed_image(fixed)
        obj = xr.PopulationObjective(rcp, [m], 100)
        poses = synth.sample_poses(w.vol, w.gt, 100, 10.0, 20.0, seed=11)
        mix = obj.eval(poses)
        for i in (0, 37, 99):
            np.testing.assert_array_equal(obj.eval(poses[i:i + 1]), mix[i:i + 1])
        perm = np.random.default_rng(1).permutation(100)
        np.testing.assert_array_equal(obj.eval(poses[perm]), mix[perm])
        vals[vt] = mix
    np.testing.assert_allclose(vals[1], vals[0], atol=1e-4, rtol=0)
