"""The benchmark's synthetic workloads restated in numpy for the checker side.

TEST INFRASTRUCTURE ONLY: the CPU baseline and the reference arm of bench.py
build their inputs here, so the timed reference path loads nothing of the
product (no xreg_gb300 import, no libxreg_gb300.so).  The generators are the
same seeded procedures as the product's own (tests/test_workload_cpu.py holds
them equal bit for bit):

* phantom: a soft-tissue body ellipsoid (base HU ~ U(0, 60) plus per-voxel
  N(0, 10^2) noise) in air (-1000 HU) holding 3-5 bone ellipsoids at
  HU ~ U(300, 1500), converted with HUToLinAtt (lib/image/xregHUToLinAtt.cpp:45-69,
  mu_water 0.02683 / mm);
* camera: the oracle's own naive camera set-up and downsampling;
* poses: rotations about the volume centre ~ N(0, sigma_deg) per axis and
  translations ~ N(0, sigma_mm), applied to the nominal view (volume centre
  700 mm from the source along the camera's -z axis).
"""
from __future__ import annotations

import numpy as np

from . import oracle as O

MU_WATER = 0.02683
MU_AIR = 0.02485e-4
SOURCE_TO_CENTRE_MM = 700.0
SDD_MM = 1020.0


def hu_to_lin_att(hu):
    hu_scale = (MU_WATER - MU_AIR) * 1.0e-3
    mu_lower = -1000.0 * hu_scale + MU_WATER
    v = hu.astype(np.float64) * hu_scale + MU_WATER - mu_lower
    return np.maximum(v, 0.0).astype(np.float32)


def phantom(size_xyz, spacing, seed: int, slab: int = 16) -> np.ndarray:
    """Attenuation volume [nz, ny, nx] of the seeded ellipsoid phantom."""
    nx, ny, nz = (int(v) for v in size_xyz)
    sp = np.asarray(spacing, dtype=np.float64)
    ext = np.array([nx, ny, nz], dtype=np.float64) * sp
    rng = np.random.default_rng(seed)
    body_c = ext / 2.0 + rng.uniform(-0.02, 0.02, 3) * ext
    body_a = ext * np.array([rng.uniform(0.40, 0.46), rng.uniform(0.30, 0.38), rng.uniform(0.42, 0.47)])
    body_hu = rng.uniform(0.0, 60.0)
    bones = []
    for _ in range(int(rng.integers(3, 6))):
        c = body_c + rng.uniform(-0.55, 0.55, 3) * body_a
        a = ext * rng.uniform(0.04, 0.14, 3)
        bones.append((c, a, rng.uniform(300.0, 1500.0)))
    noise_rng = np.random.default_rng(seed + 7919)
    hu_vol = np.empty((nz, ny, nx), dtype=np.float32)
    X, Y = np.meshgrid(np.arange(nx) * sp[0], np.arange(ny) * sp[1], indexing="xy")
    for z0 in range(0, nz, slab):
        z1 = min(nz, z0 + slab)
        Z = (np.arange(z0, z1) * sp[2])[:, None, None]

        def inside(c, a):
            return (((X[None] - c[0]) / a[0]) ** 2 + ((Y[None] - c[1]) / a[1]) ** 2 + ((Z - c[2]) / a[2]) ** 2) <= 1.0

        body = inside(body_c, body_a)
        hu = np.where(body, body_hu, -1000.0)
        for c, a, h in bones:
            hu = np.where(inside(c, a) & body, h, hu)
        noise = noise_rng.standard_normal(hu.shape, dtype=np.float32) * 10.0
        hu_vol[z0:z1] = np.where(body, hu + noise, hu).astype(np.float32)
    return hu_to_lin_att(hu_vol)


def _rigid(R, t):
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = t
    return T


def _euler_xyz(rx, ry, rz):
    cx, sx, cy, sy, cz, sz = np.cos(rx), np.sin(rx), np.cos(ry), np.sin(ry), np.cos(rz), np.sin(rz)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def centre_xform(size_xyz, spacing) -> np.ndarray:
    """RayCaster::xform_img_center_to_itk_phys (xregRayCastInterface.cpp:200-224)
    for an axis-aligned volume at the origin."""
    T = np.eye(4)
    T[:3, 3] = np.asarray(size_xyz, dtype=np.float64) / 2.0 * np.asarray(spacing, dtype=np.float64)
    return T


def gt_pose(size_xyz, spacing) -> np.ndarray:
    """Nominal view: the volume centre at camera (0, 0, -700 mm), viewed along +y."""
    R = np.array([[1.0, 0.0, 0.0], [0.0, 0.0, 1.0], [0.0, -1.0, 0.0]])
    return centre_xform(size_xyz, spacing) @ _rigid(R, R @ np.array([0.0, 0.0, SOURCE_TO_CENTRE_MM]))


def perturb(size_xyz, spacing, pose, rot_deg, trans_mm) -> np.ndarray:
    C = centre_xform(size_xyz, spacing)
    D = _rigid(_euler_xyz(*np.radians(rot_deg)), trans_mm)
    return C @ D @ np.linalg.inv(C) @ pose


def sample_poses(size_xyz, spacing, pose, n, rot_sigma_deg, trans_sigma_mm, seed) -> np.ndarray:
    rng = np.random.default_rng(seed)
    out = np.empty((n, 4, 4))
    for i in range(n):
        out[i] = perturb(size_xyz, spacing, pose, rng.normal(0.0, rot_sigma_deg, 3),
                         rng.normal(0.0, trans_sigma_mm, 3))
    return out


def add_noise(img, frac, seed):
    rng = np.random.default_rng(seed)
    return (img + rng.normal(0.0, frac * float(img.max() - img.min()), img.shape)).astype(np.float32)


class Batched:
    """The batched population workload: 256^3 phantom at 1 mm, 1536^2 detector
    at 0.194 mm downsampled 4x to 384^2, step 0.5 mm, lambda = 100,
    rotations N(0, 10 deg), translations N(0, 20 mm), grad-NCC."""

    def __init__(self, seed: int = 0, pop: int = 100):
        self.size, self.spacing, self.seed, self.pop, self.step = (256, 256, 256), (1.0, 1.0, 1.0), seed, pop, 0.5
        self.rot_sigma, self.trans_sigma = 10.0, 20.0
        self.voxels = phantom(self.size, self.spacing, seed)
        self.geom = O.vol_geom_of(self.voxels, self.spacing)
        self.cams = [O.camera_downsample(O.camera_naive(SDD_MM, 1536, 1536, 0.194, 0.194, 1), 0.25)]
        self.gt = gt_pose(self.size, self.spacing)

    def fixed_pose(self) -> np.ndarray:
        rng = np.random.default_rng(self.seed + 1)
        return perturb(self.size, self.spacing, self.gt, rng.normal(0.0, 5.0, 3), rng.normal(0.0, 10.0, 3))

    def populations(self, n: int, seed: int) -> np.ndarray:
        rng = np.random.default_rng(seed)
        return np.stack([sample_poses(self.size, self.spacing, self.gt, self.pop, self.rot_sigma, self.trans_sigma,
                                      int(rng.integers(1 << 30))) for _ in range(n)])
