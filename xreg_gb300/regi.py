"""Intensity-based 2D/3D registration driven by the GPU population objective.

A `Registration` is one job of xReg's MultiLevelMultiObjRegi for a single object
(lib/regi/interfaces_2d_3d/xregMultiObjMultiLevel2D3DRegi.cpp:164-531): a list of
levels (camera models, fixed images, metric, optimizer schedule); at each level a
CMA-ES (Intensity2D3DRegiCMAES::run, xregIntensity2D3DRegiCMAES.cpp:76-247)
searches SE(3) Lie-algebra offsets x (SE3OptVarsLieAlg, xregSE3OptVars.cpp:128-137)
applied about an intermediate frame at the volume centre, so a candidate pose is

    pose(x) = C @ ExpSE3(x) @ inv(C) @ start_pose        (C = volume centre frame),

the objective is the mean over views of the metric (one GPU population
evaluation per generation), out-of-bounds candidates are resampled, and the next
level starts from the previous level's result.

The job exposes a step interface (propose / tell) so a server can evaluate the
populations of many jobs in one GPU launch (continuous batching); `run()` drives
one job alone.  The volume is uploaded once per job and stays on the device.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import api
from .cmaes import CMAES, TrustRegionDFO

# Bounds of xReg's single-view BOBYQA level (+-2.5 deg rotations, +-5, 5, 10 mm).
DFO_BOUNDS = np.array([np.radians(2.5)] * 3 + [5.0, 5.0, 10.0])

METRICS = {
    "ncc": api.ImgSimMetric2DNCCCUDA,
    "grad_ncc": api.ImgSimMetric2DGradNCCCUDA,
    "patch_ncc": api.ImgSimMetric2DPatchNCCCUDA,
    "patch_grad_ncc": api.ImgSimMetric2DPatchGradNCCCUDA,
}

# xReg's single-view pelvis registration uses sigma (15, 15, 30 deg, 50, 50, 100 mm)
# for its first level; these are milder defaults for perturbations of ~10 deg / 20 mm.
DEFAULT_SIGMA = np.array([np.radians(10.0)] * 3 + [20.0] * 3)


@dataclass
class RegiLevel:
    cams: list                      # CameraModel per view
    fixed: list                     # fixed image per view (rows x cols float32)
    metric: str = "grad_ncc"
    pop: int = 50
    sigma: np.ndarray = field(default_factory=lambda: DEFAULT_SIGMA.copy())
    bounds: np.ndarray | None = None
    max_iters: int = 100
    tol_fun: float = 1e-6
    tol_x: float = 1e-6
    # "cmaes" (Intensity2D3DRegiCMAES) or "dfo": the bound-constrained model
    # trust region used where xReg runs NLopt's BOBYQA; for "dfo" the bounds
    # default to xReg's single-view app (+-2.5 deg, +-5/5/10 mm) and rho is in mm
    optimizer: str = "cmaes"
    rho_beg: float = 2.0
    rho_end: float = 0.01


@dataclass
class LevelResult:
    pose: np.ndarray
    x: np.ndarray
    best_value: float
    generations: int
    stop: str | None


class Registration:
    def __init__(self, vol: api.Volume, levels: list, init_pose: np.ndarray, step: float = 0.5,
                 voxel_type: int = 0, seed: int = 0, device: int = -1, name: str = "",
                 device_optimizer: bool = False):
        self.vol = vol
        self.levels = list(levels)
        self.init_pose = np.asarray(init_pose, dtype=np.float64)
        self.step = float(step)
        self.voxel_type = int(voxel_type)
        self.seed = int(seed)
        self.device = device
        self.name = name
        # CMA-ES levels keep their optimizer state in device memory, sampled and
        # updated inside the job-set step (stepped by xr_regi_jobset_step only)
        self.device_optimizer = bool(device_optimizer)
        self.C = vol.xform_img_center_to_itk_phys()
        self.Ci = np.linalg.inv(self.C)
        self.rc = None
        self.level = -1
        self.obj = None
        self.es = None
        self.start_pose = self.init_pose.copy()
        self.results: list = []
        self.done = False
        self.started = False
        self.t_submit = None
        self.t_start = None
        self.t_done = None
        self._pop_x = None

    def reset(self) -> None:
        """Back to the state before start(): the same request can be run again
        (its optimizers are seeded, so it repeats the same registration)."""
        if self.obj is not None:
            self.obj.close()
        if self.rc is not None:
            self.rc.close()
        self.rc = self.obj = self.es = None
        self.level = -1
        self.start_pose = self.init_pose.copy()
        self.results = []
        self.done = self.started = False
        self.t_submit = self.t_start = self.t_done = None
        self._pop_x = None

    # ---------------------------------------------------------- resources
    def footprint_bytes(self) -> int:
        """Device memory the job holds while active (volume copies + the largest level's buffers)."""
        nx, ny, nz = self.vol.size
        bvox = 4 if self.voxel_type == 0 else 2
        vol = nx * ny * nz * bvox + (nx - 1) * (ny - 1) * (nz - 1) * bvox * 8
        lev = 0
        for L in self.levels:
            r, c = L.cams[0].num_det_rows, L.cams[0].num_det_cols
            pop = 14 if L.optimizer == "dfo" else L.pop
            per = len(L.cams) * pop * r * c * 4 + len(L.cams) * r * c * 4 * 6 + len(L.cams) * pop * 2048 * 8
            lev = max(lev, per)
        return int(vol + lev + (16 << 20))

    def start(self) -> None:
        """Admission: the volume upload and the first level's set-up (t_start
        marks the start of the service, the end of the queue wait)."""
        self.t_start = time.perf_counter()
        self.rc = api.RayCasterLineIntCUDA(self.device)
        self.rc.set_volume(self.vol, self.voxel_type)
        self.rc.set_ray_step_size(self.step)
        self.started = True
        self._enter_level(0)

    def _enter_level(self, k: int) -> None:
        L = self.levels[k]
        self.level = k
        self.rc.set_camera_models(L.cams)
        ms = []
        for f in L.fixed:
            m = METRICS[L.metric](self.device)
            m.set_fixed_image(f)
            ms.append(m)
        if self.obj is not None:
            self.obj.close()
        if L.optimizer == "dfo":
            b = DFO_BOUNDS if L.bounds is None else np.asarray(L.bounds, dtype=np.float64)
            self.obj = api.PopulationObjective(self.rc, ms, 2 * 6 + 2)
            self.es = TrustRegionDFO(np.zeros(6), -b, b, L.rho_beg, L.rho_end, L.max_iters)
        else:
            self.obj = api.PopulationObjective(self.rc, ms, L.pop)
            self.es = CMAES(np.zeros(6), L.sigma, L.pop, seed=self.seed * 1009 + k)
            self.es.set_stop(tol_fun=L.tol_fun, tol_x=L.tol_x, max_iter=L.max_iters)
            if self.device_optimizer:
                self.es.attach_device(self.device)

    def poses_of(self, xs: np.ndarray) -> np.ndarray:
        # the library's map, so a job stepped natively (xr_regi_jobset_step)
        # sees bit-identical poses
        return api.regi_pose_map(self.C, self.start_pose, xs)

    # ---------------------------------------------------------- stepping
    def propose(self) -> np.ndarray:
        """Samples the current level's population; returns its poses [pop, 4, 4]."""
        L = self.levels[self.level]
        if L.optimizer == "dfo":
            self._pop_x = self.es.ask()
        else:
            if self.es.on_device:
                raise RuntimeError("propose: this level's optimizer lives on the device; step it with JobSet.regi_step")
            self._pop_x = self.es.sample_within_bounds(L.bounds).copy()
        return self.poses_of(self._pop_x)

    def tell(self, values) -> None:
        L = self.levels[self.level]
        if L.optimizer == "dfo":
            self.es.tell(np.asarray(values, dtype=np.float64))
        else:
            self.es.update_distribution(np.asarray(values, dtype=np.float64))
        stop = self.es.test_for_termination()
        if stop is not None:
            self.end_level(stop)

    # ----------------------------------------------------- native stepping
    def step_job(self):
        """This generation as an xr_regi_step_job for xr_regi_jobset_step (the
        optimizer advances inside the library)."""
        from ._lib import XR_REGI_CMAES, XR_REGI_DFO, xr_regi_step_job
        L = self.levels[self.level]
        j = xr_regi_step_job()
        j.obj = self.obj._h.value
        j.optimizer = XR_REGI_DFO if L.optimizer == "dfo" else XR_REGI_CMAES
        j.opt = self.es._h.value
        j.centre[:] = np.ascontiguousarray(self.C, dtype=np.float64).ravel().tolist()
        j.start_pose[:] = np.ascontiguousarray(self.start_pose, dtype=np.float64).ravel().tolist()
        b = L.bounds if (L.optimizer != "dfo" and L.bounds is not None) else np.zeros(6)
        j.bounds[:] = np.asarray(b, dtype=np.float64).ravel().tolist()
        return j

    def stop_reason(self, code: int) -> str:
        """The name of a termination code of the current level's optimizer."""
        from .cmaes import STOP_REASONS
        if self.levels[self.level].optimizer == "dfo":
            return {2: "rho_end", 3: "max_iter"}.get(code, "unknown")
        return STOP_REASONS.get(code, "unknown")

    def end_level(self, stop: str) -> None:
        """The current level has stopped (reason stop): keep its best pose, go on or finish."""
        st = self.es.state()
        x = st["best_x"]
        pose = self.poses_of(x[None])[0]
        gens = st.get("generation", st.get("iterations", 0))
        self.results.append(LevelResult(pose, x, st["best_f"], gens, stop))
        self.start_pose = pose
        if self.level + 1 < len(self.levels):
            self._enter_level(self.level + 1)
        else:
            self.finish()

    def finish(self) -> None:
        self.done = True
        self.t_done = time.perf_counter()
        if self.obj is not None:
            self.obj.close()
            self.obj = None
        if self.rc is not None:
            self.rc.close()
            self.rc = None

    @property
    def final_pose(self) -> np.ndarray:
        return self.results[-1].pose if self.results else self.init_pose

    def run(self) -> np.ndarray:
        """Runs the job alone to completion (with a device optimizer, through a
        job set of one: sampling and update stay on the device)."""
        if not self.started:
            self.start()
        js = api.JobSet(self.device) if self.device_optimizer else None
        while not self.done:
            L = self.levels[self.level]
            if js is not None and L.optimizer != "dfo":
                stop, _ = js.regi_step([self.step_job()])
                if stop[0]:
                    self.end_level(self.stop_reason(stop[0]))
                continue
            poses = self.propose()
            self.tell(self.obj.eval(poses))
        return self.final_pose


def run_level_native(obj: api.PopulationObjective, centre: np.ndarray, start_pose: np.ndarray,
                     level: RegiLevel, seed: int = 0) -> LevelResult:
    """One level run entirely in the library (xr_regi_run_level): the same loop as
    Registration's propose / tell for that level, without Python in between."""
    import ctypes as C
    from . import _lib as L
    opt = L.XR_REGI_DFO if level.optimizer == "dfo" else L.XR_REGI_CMAES
    p = L.xr_regi_level_params()
    L.call("xr_regi_level_params_default", opt, C.byref(p))
    if opt == L.XR_REGI_CMAES:
        p.lambda_ = int(level.pop)
        for i in range(6):
            p.sigma[i] = float(level.sigma[i])
            p.bounds[i] = 0.0 if level.bounds is None else float(level.bounds[i])
        p.tol_fun, p.tol_x = float(level.tol_fun), float(level.tol_x)
    else:
        b = DFO_BOUNDS if level.bounds is None else np.asarray(level.bounds, dtype=np.float64)
        for i in range(6):
            p.bounds[i] = float(b[i])
        p.rho_beg, p.rho_end = float(level.rho_beg), float(level.rho_end)
    p.max_iters = int(level.max_iters)
    p.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    c = np.ascontiguousarray(centre, dtype=np.float64)
    s = np.ascontiguousarray(start_pose, dtype=np.float64)
    out = np.zeros((4, 4))
    bf, it, why = C.c_double(), C.c_int64(), C.c_int32()
    L.call("xr_regi_run_level", obj.handle, c.ctypes.data_as(C.c_void_p), s.ctypes.data_as(C.c_void_p), C.byref(p),
           out.ctypes.data_as(C.c_void_p), C.byref(bf), C.byref(it), C.byref(why))
    return LevelResult(out, None, bf.value, it.value, why.value)


def pose_error(a: np.ndarray, b: np.ndarray, vol: api.Volume) -> tuple:
    """Difference of two cam -> ITK physical poses as (rotation angle in degrees,
    displacement in mm of the volume centre in camera coordinates)."""
    c = vol.xform_img_center_to_itk_phys()[:, 3]
    ai, bi = np.linalg.inv(a), np.linalg.inv(b)
    R = ai[:3, :3] @ bi[:3, :3].T
    ang = float(np.degrees(np.arccos(np.clip((np.trace(R) - 1.0) * 0.5, -1.0, 1.0))))
    return ang, float(np.linalg.norm((ai @ c)[:3] - (bi @ c)[:3]))
