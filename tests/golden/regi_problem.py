"""A small single-view registration level on the oracle's CPU objective, shared
by make_regi_golden.py (which records the reference's own CMA-ES on it) and
tests/test_regi_vs_reference_cpu.py (which runs the library's CMA-ES on it).

TEST INFRASTRUCTURE ONLY (numpy and the oracle): a 64x64x48 phantom at 2 mm,
one 64x64 view (the 1536^2 0.194 mm detector downsampled 24x: 4.656 mm
pixels), step 1 mm, grad-NCC with 5x5 smoothing against the DRR at the truth.
The level optimises x = (rotation vector, translation) of
pose(x) = C ExpSE3(x) C^-1 start about the volume centre C, as
Intensity2D3DRegiCMAES::run does with SE3OptVarsLieAlg (xregIntensity2D3DRegiCMAES.cpp:76-247)."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O
from oracle import workload as W

SIZE, SPACING, STEP = (64, 64, 48), (2.0, 2.0, 2.0), 1.0
LAM, SIGMA = 12, np.array([0.05, 0.05, 0.05, 6.0, 6.0, 6.0])  # radians, mm
TOL_FUN, TOL_X, MAX_ITER = 1e-7, 1e-6, 150
SEEDS = (1, 2, 3)


def exp_se3(x):
    """ExpSE3 of x = [w, v] (xregRigidUtils.cpp:40-85)."""
    w, v = np.asarray(x[:3], dtype=np.float64), np.asarray(x[3:], dtype=np.float64)
    th = float(np.sqrt(w @ w))
    W_ = np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])
    if th > 1e-14:
        a, b, c = np.sin(th) / th, (1 - np.cos(th)) / th ** 2, (th - np.sin(th)) / th ** 3
        R = np.eye(3) + a * W_ + b * W_ @ W_
        V = np.eye(3) + b * W_ + c * W_ @ W_
    else:
        R, V = np.eye(3), np.eye(3)
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = V @ v
    return T


class Problem:
    def __init__(self):
        self.voxels = W.phantom(SIZE, SPACING, 7)
        self.geom = O.vol_geom_of(self.voxels, SPACING)
        self.cam = O.camera_downsample(O.camera_naive(W.SDD_MM, 1536, 1536, 0.194, 0.194, 1), 1.0 / 24.0)
        self.truth = W.gt_pose(SIZE, SPACING)
        self.C = W.centre_xform(SIZE, SPACING)
        self.start = W.perturb(SIZE, SPACING, self.truth, [2.0, -1.5, 2.5], [4.0, -3.0, 5.0])
        self.B = np.linalg.inv(self.C) @ self.start
        self.fixed = O.drr_f32(self.voxels, self.geom, [self.cam], self.truth[None], step=STEP)[0]

    def poses(self, xs):
        return np.stack([self.C @ exp_se3(x) @ self.B for x in np.atleast_2d(xs)])

    def values(self, xs):
        drr = O.drr_f32(self.voxels, self.geom, [self.cam], self.poses(xs), step=STEP)
        return O.grad_ncc(self.fixed, drr, smooth_ksize=5)

    def error(self, x, other=None):
        """Rotation angle (deg) between pose(x) and the truth (or another pose),
        and the displacement (mm) of the volume centre in camera coordinates."""
        a, b = np.linalg.inv(self.poses(x)[0]), np.linalg.inv(self.truth if other is None else other)
        R = a[:3, :3] @ b[:3, :3].T
        ang = float(np.degrees(np.arccos(np.clip((np.trace(R) - 1.0) * 0.5, -1.0, 1.0))))
        c = self.C[:, 3]
        return ang, float(np.linalg.norm((a @ c)[:3] - (b @ c)[:3]))
