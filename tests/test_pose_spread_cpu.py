"""The pose-spread estimates that gate pose-grouped DRR items in a job-set step
(xr_posespread.h), compiled for the host as the library is, against numpy:
identical poses spread 0, a translation by delta spreads |delta| / min spacing,
random populations on an oriented anisotropic volume match the largest corner
displacement computed with numpy's general inverse, and the device
optimizer's bound is 3 (sd_trans + sd_rot * half diagonal) / min spacing."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from xreg_gb300 import synth
from xreg_gb300.se3 import euler_xyz

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = tmp_path_factory.mktemp("spread") / "pose_spread_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", f"-I{ROOT / 'xreg_gb300' / 'csrc'}",
                    f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp/pose_spread_check.cpp"), "-o", str(out)],
                   check=True)
    return out


def _run(exe, vol, poses, sd_rot, sd_trans, tmp_path):
    head = np.concatenate([np.array(vol.voxels.shape[::-1], dtype=np.float64), np.asarray(vol.spacing, np.float64),
                           np.asarray(vol.origin, np.float64), np.asarray(vol.direction, np.float64).ravel(),
                           [len(poses), sd_rot, sd_trans]])
    fi, fo = tmp_path / "in.f64", tmp_path / "out.f64"
    np.concatenate([head, np.asarray(poses, np.float64).ravel()]).tofile(fi)
    subprocess.run([str(exe), str(fi), str(fo)], check=True)
    return np.fromfile(fo, dtype=np.float64)


def _numpy_spread(vol, poses):
    n = np.array(vol.voxels.shape[::-1])
    idx = np.array([[(c >> b) & 1 for b in range(3)] for c in range(8)]) * (n - 1)
    phys = np.asarray(vol.origin) + (np.asarray(vol.direction) @ (idx * np.asarray(vol.spacing)).T).T
    h = np.concatenate([phys, np.ones((8, 1))], axis=1)
    cam = [(np.linalg.inv(p) @ h.T).T[:, :3] for p in poses]
    return max(np.linalg.norm(c - cam[0], axis=1).max() for c in cam) / min(vol.spacing)


def test_pose_spread(exe, tmp_path):
    vol = synth.phantom_volume((40, 36, 30), (0.8, 1.1, 1.6), 3)
    vol.direction = euler_xyz(0.2, -0.1, 0.4)
    gt = synth.gt_pose(vol)
    got = _run(exe, vol, np.stack([gt, gt, gt]), 0.0, 0.0, tmp_path)
    assert got[0] == 0.0 and got[1] == 0.0
    shifted = gt.copy()
    shifted[:3, 3] += [0.3, -0.4, 0.0]
    got = _run(exe, vol, np.stack([gt, shifted]), 0.0, 0.0, tmp_path)
    assert abs(got[0] - 0.5 / 0.8) < 1e-9
    for spread, seed in (((0.02, 0.05), 1), ((1.0, 2.0), 2), ((10.0, 20.0), 3)):
        poses = synth.sample_poses(vol, gt, 9, *spread, seed=seed)
        got = _run(exe, vol, poses, 0.01, 0.2, tmp_path)
        np.testing.assert_allclose(got[0], _numpy_spread(vol, poses), rtol=1e-9)
        half = 0.5 * np.array(vol.voxels.shape[::-1]) * np.asarray(vol.spacing)
        np.testing.assert_allclose(got[1], 3.0 * (0.2 + 0.01 * np.linalg.norm(half)) / 0.8, rtol=1e-12)
