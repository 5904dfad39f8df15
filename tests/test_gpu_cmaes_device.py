"""CMA-ES with its state in device memory (xr_cmaes_attach_device), sampled
inside the job-set geometry launch and updated behind the batched grad-NCC
launch, against the same optimizer on the host.

Host and device run one source (xr_cmaes_core.h) with one rounding per
operation, so after every generation the whole state block (distribution,
paths, covariance and its eigen-decomposition, last population and its draws,
history) is identical byte for byte, with and without bound redraws and on
both job-set steps; a whole registration gives the identical final pose; the
step stays at three launches (geometry + sampling, DRR, grad-NCC + update); a
job whose metric is not grad-NCC is updated by one extra launch; a candidate
that cannot be drawn inside its bounds is reported as an error."""
import numpy as np
import pytest

from tests.helpers import oracle_cams, oracle_geom, small_camera, small_volume
from xreg_gb300 import synth

pytestmark = pytest.mark.gpu


def _objective(xr, vol, cams, fixed, lam, kind=None):
    rc = xr.RayCasterLineIntCUDA()
    rc.set_volume(vol, 0)
    rc.set_camera_models(cams)
    rc.set_ray_step_size(0.5)
    ms = []
    for f in fixed:
        m = (kind or xr.ImgSimMetric2DGradNCCCUDA)()
        m.set_fixed_image(f)
        ms.append(m)
    return xr.PopulationObjective(rc, ms, lam)


def _step_job(obj, es, C, start, bounds):
    from xreg_gb300 import _lib as L
    j = L.xr_regi_step_job()
    j.obj = obj._h.value
    j.optimizer = L.XR_REGI_CMAES
    j.opt = es._h.value
    j.centre[:] = np.ascontiguousarray(C, dtype=np.float64).ravel().tolist()
    j.start_pose[:] = np.ascontiguousarray(start, dtype=np.float64).ravel().tolist()
    j.bounds[:] = list(bounds)
    return j


def _setup(xr, oracle, lam, kind=None, nviews=1):
    vol = small_volume(21, (44, 40, 36), (1.5, 1.5, 1.5))
    cams = [small_camera((40, 44), 3.0) for _ in range(nviews)]
    gt = synth.gt_pose(vol)
    fixed = [f for f in oracle.drr_f32(vol.voxels, oracle_geom(vol), oracle_cams(cams), np.stack([gt] * nviews),
                                       cam_idx=list(range(nviews)), step=0.5)]
    start = synth.perturb(vol, gt, (2.0, -3.0, 1.5), (4.0, -2.0, 5.0))
    C = vol.xform_img_center_to_itk_phys()
    return vol, cams, fixed, C, start, [_objective(xr, vol, cams, fixed, lam, kind) for _ in range(2)]


@pytest.mark.parametrize("bounds,fused", [((0.0,) * 6, False), ((0.06, 0.06, 0.06, 6.0, 6.0, 6.0), False),
                                          ((0.06, 0.06, 0.06, 6.0, 6.0, 6.0), True)])
def test_device_state_equals_host_every_generation(xr, oracle, bounds, fused):
    from xreg_gb300.cmaes import CMAES
    lam = 12
    vol, cams, fixed, C, start, (obj_h, obj_d) = _setup(xr, oracle, lam)
    sigma = [0.1, 0.1, 0.1, 8.0, 8.0, 8.0]
    es_h, es_d = CMAES(np.zeros(6), sigma, lam, seed=77), CMAES(np.zeros(6), sigma, lam, seed=77)
    for es in (es_h, es_d):
        es.set_stop(tol_fun=1e-9, tol_x=1e-7, max_iter=25)
    es_d.attach_device()
    js = xr.JobSet()
    js.set_fused(fused)
    gens = 0
    for g in range(25):
        stop, ev = js.regi_step([_step_job(obj_h, es_h, C, start, bounds), _step_job(obj_d, es_d, C, start, bounds)])
        assert ev == [lam, lam]
        assert es_h.export_state() == es_d.export_state(), f"generation {g}"
        assert stop[0] == stop[1]
        gens += 1
        if stop[0]:
            break
    st = es_d.state()
    assert st["generation"] == gens and np.isfinite(st["best_f"])
    es_d.detach_device()
    assert es_d.export_state() == es_h.export_state()


def test_launches_and_other_metrics(xr, oracle):
    from xreg_gb300.cmaes import CMAES
    lam = 8
    vol, cams, fixed, C, start, (obj_a, obj_b) = _setup(xr, oracle, lam)
    _, _, _, _, _, (ncc_h, ncc_d) = _setup(xr, oracle, lam, xr.ImgSimMetric2DNCCCUDA)
    sig = [0.1, 0.1, 0.1, 8.0, 8.0, 8.0]
    b = (0.0,) * 6
    es = [CMAES(np.zeros(6), sig, lam, seed=5) for _ in range(4)]
    es[1].attach_device()
    es[3].attach_device()
    js = xr.JobSet()
    # grad-NCC with a device optimizer: geometry + sampling, DRR, grad-NCC + update
    for _ in range(2):
        js.regi_step([_step_job(obj_b, es[1], C, start, b)])
    assert js.last_kernel_launches() == 3
    # a host optimizer beside it adds no launch
    js.regi_step([_step_job(obj_a, es[0], C, start, b), _step_job(obj_b, es[1], C, start, b)])
    assert js.last_kernel_launches() == 3
    # NCC jobs: their metric launches after the DRR; a device optimizer adds its update launch
    js.regi_step([_step_job(ncc_h, es[2], C, start, b)])
    host_launches = js.last_kernel_launches()
    js.regi_step([_step_job(ncc_d, es[3], C, start, b)])
    assert js.last_kernel_launches() == host_launches + 1
    # and its state follows the host optimizer's bit for bit
    es2 = CMAES(np.zeros(6), sig, lam, seed=5)
    es3 = CMAES(np.zeros(6), sig, lam, seed=5)
    es3.attach_device()
    for _ in range(4):
        js.regi_step([_step_job(ncc_h, es2, C, start, b), _step_job(ncc_d, es3, C, start, b)])
        assert es2.export_state() == es3.export_state()


def test_refusals_and_sampling_error(xr, oracle):
    from xreg_gb300 import _lib
    from xreg_gb300.cmaes import CMAES
    lam = 4
    vol, cams, fixed, C, start, (obj, _) = _setup(xr, oracle, lam)
    es = CMAES(np.zeros(6), [0.5, 0.5, 0.5, 30.0, 30.0, 30.0], lam, seed=1)
    es.attach_device()
    with pytest.raises(_lib.XRegError):
        es.sample_population()
    with pytest.raises(_lib.XRegError):
        es.update_distribution(np.zeros(lam))
    with pytest.raises(_lib.XRegError):
        es.set_stop(1e-6, 1e-6, 10)
    assert es.test_for_termination() is None and es.state()["generation"] == 0
    # bounds no draw can meet: every candidate gives up after the redraw limit
    js = xr.JobSet()
    with pytest.raises(_lib.XRegError, match="inside the bounds"):
        js.regi_step([_step_job(obj, es, C, start, (1e-12,) * 6)])
    # the same handle back on the host samples again
    es2 = CMAES(np.zeros(6), [0.5, 0.5, 0.5, 30.0, 30.0, 30.0], lam, seed=1)
    es2.attach_device()
    es2.detach_device()
    assert es2.sample_population().shape == (lam, 6)


def test_registration_with_device_optimizer_equals_host(xr):
    """A whole two-level registration (CMA-ES then the trust region) run with
    the CMA-ES state on the device ends at the bit-identical pose."""
    spec = synth.JobSpec(seed=4, size=(96, 96, 80), spacing=(2.0, 2.0, 2.0), view_angles=[0.0, 30.0], ds_first=0.125,
                         pop=16)
    host, _ = synth.job_registration(spec, iters=(30, 10), level2_pop=6)
    dev, _ = synth.job_registration(spec, iters=(30, 10), level2_pop=6)
    dev.device_optimizer = True
    p_h = host.run()
    p_d = dev.run()
    np.testing.assert_array_equal(p_h, p_d)
    for a, b in zip(host.results, dev.results):
        assert a.best_value == b.best_value and a.generations == b.generations and a.stop == b.stop
