"""Registration and serving on the GPU.

* A two-level registration (CMA-ES at 8x, then the bound-constrained trust
  region at 4x, grad-NCC, fixed images downsampled from full-resolution DRRs)
  of a seeded two-view phantom recovers the ground-truth pose within
  0.05 deg / 0.1 mm.
* The continuous-batching server gives every job exactly the result it gets
  when run alone (its optimizer has its own random stream and the job-set values
  equal the single-job values), while several jobs share each GPU step, whether
  the generation is stepped in the library (xr_regi_jobset_step) or from Python.
"""
import numpy as np
import pytest

from xreg_gb300 import synth
from xreg_gb300.regi import pose_error

pytestmark = pytest.mark.gpu


def _spec(seed, size=(128, 128, 96), views=(0.0,), ds=0.125, pop=24):
    return synth.JobSpec(seed=seed, size=size, spacing=(2.0, 2.0, 2.0), view_angles=list(views), ds_first=ds,
                         pop=pop)


def test_two_level_registration_recovers_pose(xr):
    job, gt = synth.job_registration(_spec(3, views=(0.0, 30.0)), iters=(80, 40), level2_pop=10)
    err0 = pose_error(job.init_pose, gt, job.vol)
    pose = job.run()
    rot, trans = pose_error(pose, gt, job.vol)
    assert err0[0] > 2.0 or err0[1] > 5.0  # it started away from the truth
    print(f"start error {err0[0]:.3f} deg / {err0[1]:.3f} mm -> final {rot:.4f} deg / {trans:.4f} mm")
    # the registration tolerance the path is specified with: 0.05 deg / 0.1 mm
    assert rot < 0.05 and trans < 0.1, (rot, trans, err0)
    assert len(job.results) == 2 and job.results[1].best_value <= job.results[0].best_value + 0.05


@pytest.mark.parametrize("native_step", [True, False])
def test_server_results_equal_alone(xr, native_step):
    """native_step: each generation of all jobs in one xr_regi_jobset_step call;
    otherwise sampled and updated from Python.  Both give the alone results."""
    from xreg_gb300.serving import RegistrationServer
    specs = [_spec(10 + k, size=s, views=v, ds=d, pop=p) for k, (s, v, d, p) in enumerate([
        ((96, 96, 80), (0.0,), 0.125, 16), ((128, 112, 96), (0.0, 25.0), 0.125, 20),
        ((112, 128, 100), (0.0, 20.0, 45.0), 0.25, 12), ((80, 96, 96), (0.0,), 0.25, 18)])]
    alone = []
    for s in specs:
        job, _ = synth.job_registration(s, iters=(25, 10), level2_pop=6)
        alone.append(job.run())
    srv = RegistrationServer(hbm_budget_bytes=180e9, native_step=native_step)
    jobs = []
    for s in specs:
        job, _ = synth.job_registration(s, iters=(25, 10), level2_pop=6)
        jobs.append(job)
    # staggered arrivals: two now, two after the first steps
    srv.submit(jobs[0])
    srv.submit(jobs[1])
    srv.step()
    srv.step()
    srv.submit(jobs[2])
    srv.submit(jobs[3])
    while srv.queue or srv.active or srv.starting:
        srv.step()
    st = srv.stats.summary()
    assert st["completed"] == 4 and st["max_active"] >= 3
    for a, j in zip(alone, jobs):
        np.testing.assert_array_equal(j.final_pose, a)


def test_server_admission_respects_budget(xr):
    from xreg_gb300.serving import RegistrationServer
    jobs = [synth.job_registration(_spec(30 + k, size=(64, 64, 64), pop=8), iters=(3, 2), level2_pop=4)[0]
            for k in range(3)]
    one = jobs[0].footprint_bytes()
    srv = RegistrationServer(hbm_budget_bytes=1.5 * one)
    for j in jobs:
        srv.submit(j)
    srv.step()
    assert len(srv.active) == 1 and len(srv.queue) == 2  # only one fits
    while srv.queue or srv.active or srv.starting:
        srv.step()
    assert srv.stats.completed == 3 and srv.stats.max_active == 1


def test_reset_repeats_the_registration(xr):
    job, _ = synth.job_registration(_spec(41, size=(64, 64, 64), pop=8), iters=(6, 4), level2_pop=4)
    first = job.run().copy()
    job.reset()
    assert not job.done and job.results == []
    np.testing.assert_array_equal(job.run(), first)


def test_native_level_driver(xr):
    """xr_regi_run_level runs a CMA-ES level and a trust-region level in the
    library and lands where the Python level loop lands (both near the truth)."""
    from xreg_gb300 import api
    from xreg_gb300.regi import run_level_native
    job, gt = synth.job_registration(_spec(3, views=(0.0, 30.0)), iters=(80, 40), level2_pop=10)
    py_pose = job.run()
    rc = api.RayCasterLineIntCUDA()
    rc.set_volume(job.vol, job.voxel_type)
    rc.set_ray_step_size(job.step)
    start = job.init_pose
    for k, L in enumerate(job.levels):
        rc.set_camera_models(L.cams)
        ms = []
        for f in L.fixed:
            m = api.ImgSimMetric2DGradNCCCUDA()
            m.set_fixed_image(f)
            ms.append(m)
        obj = api.PopulationObjective(rc, ms, 14 if L.optimizer == "dfo" else L.pop)
        res = run_level_native(obj, job.C, start, L, seed=job.seed * 1009 + k)
        start = res.pose
        obj.close()
    rot, trans = pose_error(start, gt, job.vol)
    assert rot < 0.05 and trans < 0.1, (rot, trans)
    rot2, trans2 = pose_error(start, py_pose, job.vol)
    assert rot2 < 0.05 and trans2 < 0.1, (rot2, trans2)
