"""Seeded synthetic registration workloads (phantoms, cameras, poses, fixed images).

No public dataset is named for this path; these stand in for the CT / X-ray data
xReg's walkthroughs download.  Shapes, spacings and value distributions follow
the workload definitions:

* phantom: a soft-tissue body ellipsoid (base HU ~ U(0, 60) plus per-voxel
  N(0, 10^2) noise) in air (-1000 HU), holding 3-5 bone ellipsoids at
  HU ~ U(300, 1500); HU -> attenuation with xReg's HUToLinAtt
  (lib/image/xregHUToLinAtt.cpp:45-69, mu_water 0.02683 / mm);
* camera: naive pinhole, source-to-detector 1020 mm, volume centre 700 mm from
  the source;
* poses: rotations about the volume centre ~ N(0, sigma_deg) per axis and
  translations ~ N(0, sigma_mm);
* fixed image: DRR at the ground-truth pose plus Gaussian noise with sigma = 1%
  of the DRR range.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .api import CameraModel, Volume
from .se3 import euler_xyz, rigid

MU_WATER = 0.02683
MU_AIR = 0.02485e-4
SOURCE_TO_CENTRE_MM = 700.0
SDD_MM = 1020.0


def hu_to_lin_att(hu: np.ndarray, hu_lower: float = -1000.0) -> np.ndarray:
    """HUToLinAttFilter::GenerateData: max(hu*scale + mu_w - mu_lower, 0) in double, stored as float."""
    hu_scale = (MU_WATER - MU_AIR) * 1.0e-3
    mu_lower = hu_lower * hu_scale + MU_WATER
    v = hu.astype(np.float64) * hu_scale + MU_WATER - mu_lower
    return np.maximum(v, 0.0).astype(np.float32)


def phantom_hu(size_xyz, spacing, seed: int, slab: int = 16) -> np.ndarray:
    """HU volume [nz, ny, nx] from one seed (deterministic, generated slab by slab)."""
    nx, ny, nz = (int(v) for v in size_xyz)
    sp = np.asarray(spacing, dtype=np.float64)
    ext = np.array([nx, ny, nz], dtype=np.float64) * sp
    rng = np.random.default_rng(seed)
    body_c = ext / 2.0 + rng.uniform(-0.02, 0.02, 3) * ext
    body_a = ext * np.array([rng.uniform(0.40, 0.46), rng.uniform(0.30, 0.38), rng.uniform(0.42, 0.47)])
    body_hu = rng.uniform(0.0, 60.0)
    nb = int(rng.integers(3, 6))
    bones = []
    for _ in range(nb):
        c = body_c + rng.uniform(-0.55, 0.55, 3) * body_a
        a = ext * rng.uniform(0.04, 0.14, 3)
        bones.append((c, a, rng.uniform(300.0, 1500.0)))
    noise_rng = np.random.default_rng(seed + 7919)
    out = np.empty((nz, ny, nx), dtype=np.float32)
    xs = (np.arange(nx) + 0.0) * sp[0]
    ys = (np.arange(ny) + 0.0) * sp[1]
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    for z0 in range(0, nz, slab):
        z1 = min(nz, z0 + slab)
        zs = np.arange(z0, z1) * sp[2]
        Z = zs[:, None, None]
        body = (((X[None] - body_c[0]) / body_a[0]) ** 2 + ((Y[None] - body_c[1]) / body_a[1]) ** 2 +
                ((Z - body_c[2]) / body_a[2]) ** 2) <= 1.0
        hu = np.where(body, body_hu, -1000.0)
        for c, a, h in bones:
            inb = (((X[None] - c[0]) / a[0]) ** 2 + ((Y[None] - c[1]) / a[1]) ** 2 + ((Z - c[2]) / a[2]) ** 2) <= 1.0
            hu = np.where(inb & body, h, hu)
        noise = noise_rng.standard_normal(hu.shape, dtype=np.float32) * 10.0
        hu = np.where(body, hu + noise, hu)
        out[z0:z1] = hu.astype(np.float32)
    return out


def phantom_volume(size_xyz, spacing, seed: int) -> Volume:
    hu = phantom_hu(size_xyz, spacing, seed)
    return Volume(hu_to_lin_att(hu), spacing=tuple(float(s) for s in spacing))


# camera frame: the -z axis points from the source to the detector; the volume
# is viewed along its +y axis (anterior-posterior) at the identity pose.
_R_VIEW = np.array([[1.0, 0.0, 0.0], [0.0, 0.0, 1.0], [0.0, -1.0, 0.0]])


def view_rotation(angle_deg: float) -> np.ndarray:
    """Rotation of the view about the volume's z axis (C-arm orbit) by angle_deg."""
    a = np.radians(angle_deg)
    return np.array([[np.cos(a), -np.sin(a), 0.0], [np.sin(a), np.cos(a), 0.0], [0.0, 0.0, 1.0]])


def gt_pose(vol: Volume, view_angle_deg: float = 0.0, src_to_centre: float = SOURCE_TO_CENTRE_MM) -> np.ndarray:
    """cam -> ITK physical transform placing the volume centre at camera (0, 0, -src_to_centre)."""
    R = view_rotation(view_angle_deg) @ _R_VIEW
    X = rigid(R, R @ np.array([0.0, 0.0, src_to_centre]))
    return vol.xform_img_center_to_itk_phys() @ X


def perturb(vol: Volume, pose: np.ndarray, rot_deg, trans_mm) -> np.ndarray:
    """Applies a rotation (Euler x-y-z, degrees) and translation (mm) about the volume centre."""
    C = vol.xform_img_center_to_itk_phys()
    Ci = np.linalg.inv(C)
    D = rigid(euler_xyz(*np.radians(rot_deg)), trans_mm)
    return C @ D @ Ci @ pose


def sample_poses(vol: Volume, pose: np.ndarray, n: int, rot_sigma_deg: float, trans_sigma_mm: float,
                 seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    out = np.empty((n, 4, 4))
    for i in range(n):
        out[i] = perturb(vol, pose, rng.normal(0.0, rot_sigma_deg, 3), rng.normal(0.0, trans_sigma_mm, 3))
    return out


def add_noise(img: np.ndarray, frac: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    rngv = float(img.max() - img.min())
    return (img + rng.normal(0.0, frac * rngv, img.shape)).astype(np.float32)


@dataclass
class Workload:
    name: str
    vol: Volume
    cams: list
    step: float
    gt: np.ndarray            # ground-truth cam -> ITK physical pose (view 0 frame)
    metric: str               # "ncc" | "grad_ncc" | "patch_grad_ncc"
    pop: int
    rot_sigma: float
    trans_sigma: float
    seed: int


def camera_for(det_px: int, pixel_mm: float, ds: float = 1.0) -> CameraModel:
    cam = CameraModel.naive(SDD_MM, det_px, det_px, pixel_mm, pixel_mm)
    return cam.downsample(ds) if ds != 1.0 else cam


def plain_small(seed: int = 0) -> Workload:
    """128^3 at 1.5 mm, 256^2 detector at 1.55 mm, 0.5 mm step, NCC, one pose."""
    vol = phantom_volume((128, 128, 128), (1.5, 1.5, 1.5), seed)
    return Workload("plain-128^3-256^2-ncc", vol, [camera_for(256, 1.55)], 0.5, gt_pose(vol), "ncc", 1, 5.0, 10.0,
                    seed)


def batched_population(seed: int = 0, pop: int = 100) -> Workload:
    """256^3 at 1 mm, 1536^2 at 0.194 mm downsampled 4x to 384^2, lambda = 100, grad-NCC."""
    vol = phantom_volume((256, 256, 256), (1.0, 1.0, 1.0), seed)
    return Workload("batched-256^3-384^2-gradncc-pop100", vol, [camera_for(1536, 0.194, 0.25)], 0.5, gt_pose(vol),
                    "grad_ncc", pop, 10.0, 20.0, seed)


def precision_large(seed: int = 0) -> Workload:
    """512x512x400 at 0.8x0.8x1 mm, 2x-downsampled detector (768^2), patch grad-NCC 11x11."""
    vol = phantom_volume((512, 512, 400), (0.8, 0.8, 1.0), seed)
    return Workload("precision-512x512x400-768^2-patchgradncc", vol, [camera_for(1536, 0.194, 0.5)], 0.5,
                    gt_pose(vol), "patch_grad_ncc", 1, 5.0, 10.0, seed)


def fixed_pose(w: Workload) -> np.ndarray:
    """Ground-truth pose: the nominal view perturbed by rot ~ N(0, 5 deg), trans ~ N(0, 10 mm)."""
    rng = np.random.default_rng(w.seed + 1)
    return perturb(w.vol, w.gt, rng.normal(0.0, 5.0, 3), rng.normal(0.0, 10.0, 3))


# ------------------------------------------------------------ uneven jobs
@dataclass
class JobSpec:
    """One registration request of the uneven multi-job / serving workloads."""
    seed: int
    size: tuple            # volume (nx, ny, nz)
    spacing: tuple
    view_angles: list      # degrees about the volume's z axis, one per view
    ds_first: float        # detector downsample factor of the first level (0.125 = 8x)
    pop: int


def uneven_job_specs(n: int, seed: int) -> list:
    """n requests with volumes from 192^3 to 512x512x300 (each its own seed), 1-3
    views 15-40 degrees apart, detector 1536^2 @ 0.194 mm downsampled 4x or 8x,
    CMA-ES lambda in [20, 100]."""
    rng = np.random.default_rng(seed)
    sizes = [(192, 192, 192), (256, 256, 200), (256, 256, 256), (320, 320, 256), (384, 384, 280),
             (448, 448, 300), (512, 512, 300)]
    out = []
    for k in range(n):
        size = sizes[int(rng.integers(len(sizes)))]
        sp = 300.0 / size[0]
        nv = int(rng.integers(1, 4))
        angles = [0.0]
        for _ in range(nv - 1):
            angles.append(angles[-1] + float(rng.uniform(15.0, 40.0)))
        out.append(JobSpec(seed=seed * 1000 + k, size=size, spacing=(sp, sp, sp), view_angles=angles,
                           ds_first=float(rng.choice([0.25, 0.125])), pop=int(rng.integers(20, 101))))
    return out


def job_registration(spec: JobSpec, levels=None, iters=(150, 100), level2_pop: int = 8, voxel_type: int = 1,
                     step: float = 0.5, device: int = -1, level2: str = "dfo", fixed_from: str = "downsample"):
    """A two-level registration request from a JobSpec: level 1 at the spec's
    downsampling (or 8x) with CMA-ES lambda = spec.pop, level 2 at 4x with the
    bound-constrained trust-region optimizer (level2 "dfo", xReg's BOBYQA level)
    or a small CMA-ES (level2 "cmaes", lambda = level2_pop).  The fixed images are
    full-resolution (1536^2) DRRs at a ground-truth pose plus 1 % noise, brought
    to each level by DownsampleProjData as MultiLevelMultiObjRegi does
    (xregMultiObjMultiLevel2D3DRegi.cpp:254; fixed_from "render" instead renders
    each level directly).  Start pose perturbed from the ground truth by
    N(0, 5 deg) / N(0, 10 mm).  Returns (Registration, ground truth)."""
    from .regi import Registration, RegiLevel
    vol = phantom_volume(spec.size, spec.spacing, spec.seed)
    rng = np.random.default_rng(spec.seed + 1)
    gt = perturb(vol, gt_pose(vol), rng.normal(0.0, 3.0, 3), rng.normal(0.0, 5.0, 3))
    init = perturb(vol, gt, rng.normal(0.0, 5.0, 3), rng.normal(0.0, 10.0, 3))
    ds = levels or [spec.ds_first, 0.25]
    full = None
    if fixed_from == "downsample":
        full = render_fixed(vol, view_cameras(spec.view_angles, 1.0), gt, step, spec.seed + 17, device)
    lv = []
    for k, d in enumerate(ds):
        cams = view_cameras(spec.view_angles, d)
        if full is not None:
            from .api import downsample_image
            fixed = [downsample_image(f, d, device) for f in full]
        else:
            fixed = render_fixed(vol, cams, gt, step, spec.seed + 17 * (k + 1), device)
        if k == 0:
            lv.append(RegiLevel(cams, fixed, "grad_ncc", pop=spec.pop, max_iters=iters[0]))
        elif level2 == "dfo":
            lv.append(RegiLevel(cams, fixed, "grad_ncc", optimizer="dfo", max_iters=iters[min(k, len(iters) - 1)]))
        else:
            sig = np.array([np.radians(1.5)] * 3 + [3.0] * 3)
            lv.append(RegiLevel(cams, fixed, "grad_ncc", pop=level2_pop, sigma=sig,
                                max_iters=iters[min(k, len(iters) - 1)]))
    return Registration(vol, lv, init, step=step, voxel_type=voxel_type, seed=spec.seed, device=device,
                        name=f"job{spec.seed}"), gt


def request_like(template, gt: np.ndarray, seed: int):
    """Another registration request of the same patient and views as template
    (its volume, cameras and fixed images shared), with its own start pose,
    perturbed from the ground truth by N(0, 5 deg) / N(0, 10 mm), and its own
    optimizer seed."""
    from .regi import Registration
    rng = np.random.default_rng(seed)
    init = perturb(template.vol, gt, rng.normal(0.0, 5.0, 3), rng.normal(0.0, 10.0, 3))
    return Registration(template.vol, template.levels, init, step=template.step, voxel_type=template.voxel_type,
                        seed=seed, device=template.device, name=f"{template.name}-r{seed}")


def view_cameras(angles, ds: float) -> list:
    """One naive camera per view; view k orbits angles[k] degrees about the volume centre."""
    from .se3 import rigid
    cams = []
    for a in angles:
        cam = camera_for(1536, 0.194, ds)
        if a != 0.0:
            R = np.array([[np.cos(np.radians(a)), 0.0, np.sin(np.radians(a))], [0.0, 1.0, 0.0],
                          [-np.sin(np.radians(a)), 0.0, np.cos(np.radians(a))]])
            c = np.array([0.0, 0.0, -SOURCE_TO_CENTRE_MM])
            cam.set_extrins(rigid(R, c - R @ c))
        cams.append(cam)
    return cams


def render_fixed(vol: Volume, cams: list, pose: np.ndarray, step: float, noise_seed: int, device: int = -1):
    """Fixed images: DRR of each view at the ground-truth pose (GPU ray caster) plus 1 % noise."""
    from .api import RayCasterLineIntCUDA
    rc = RayCasterLineIntCUDA(device)
    rc.set_volume(vol)
    rc.set_camera_models(cams)
    rc.set_ray_step_size(step)
    rc.set_num_projs(len(cams))
    rc.allocate_resources()
    rc.distribute_xforms_among_cam_models(pose[None])
    rc.compute()
    imgs = rc.projs()
    rc.close()
    return [add_noise(imgs[v], 0.01, noise_seed + v) for v in range(len(cams))]
