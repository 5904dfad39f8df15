"""The header-only C++ host classes (include/xreg_gb300/xreg_gb300.hpp) compile
against the C ABI and give the oracle's results when driven like xReg drives its
ray caster and metrics."""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from tests.helpers import drr_rel_err, oracle_cams, oracle_geom
from xreg_gb300 import synth

ROOT = Path(__file__).resolve().parents[1]


def _compile(tmp: Path) -> Path:
    from xreg_gb300.build import LIB_PATH
    exe = tmp / "host_api_check"
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    subprocess.run([cxx, "-std=c++17", "-O1", f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp/host_api_check.cpp"),
                    "-o", str(exe), f"-L{LIB_PATH.parent}", "-lxreg_gb300", f"-Wl,-rpath,{LIB_PATH.parent}"],
                   check=True)
    return exe


def test_cpp_header_compiles(xr, tmp_path):
    _compile(tmp_path)


@pytest.mark.gpu
def test_cpp_host_classes_match_oracle(xr, oracle, tmp_path):
    exe = _compile(tmp_path)
    vol = synth.phantom_volume((36, 40, 32), (2.0, 2.0, 2.0), 4)
    rows, cols, px, step = 30, 34, 4.0, 0.5
    poses = synth.sample_poses(vol, synth.gt_pose(vol), 4, 6.0, 8.0, seed=3)
    cam = xr.CameraModel.naive(synth.SDD_MM, rows, cols, px, px)
    fixed = synth.add_noise(oracle.drr_f32(vol.voxels, oracle_geom(vol), oracle_cams([cam]),
                                           synth.gt_pose(vol)[None], step=step)[0], 0.01, 1)
    nz, ny, nx = vol.voxels.shape
    np.array([nx, ny, nz, 2.0, rows, cols, px, step, len(poses)], np.float64).tofile(tmp_path / "meta.f64")
    vol.voxels.tofile(tmp_path / "vol.f32")
    poses.astype(np.float64).tofile(tmp_path / "poses.f64")
    fixed.tofile(tmp_path / "fixed.f32")
    mask = (np.random.default_rng(7).random((rows, cols)) > 0.3).astype(np.uint8)
    mask.tofile(tmp_path / "mask.u8")
    F = synth.perturb(vol, np.eye(4), [0.0, 3.0, 1.0], [2.0, 0.0, -1.0])
    R = synth.perturb(vol, np.eye(4), [1.0, 0.0, 0.0], [0.0, 1.5, 0.0])
    np.concatenate([F.ravel(), R.ravel()]).astype(np.float64).tofile(tmp_path / "frames.f64")
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    drr = np.fromfile(tmp_path / "drr.f32", np.float32).reshape(len(poses), rows, cols)
    sims = np.fromfile(tmp_path / "sims.f32", np.float32)
    obj = np.fromfile(tmp_path / "obj.f32", np.float32)
    ref = oracle.drr_f32(vol.voxels, oracle_geom(vol), oracle_cams([cam]), poses, step=step)
    rel, zero = drr_rel_err(drr, ref)
    assert zero == 0.0 and rel <= 1e-4
    ref_sims = oracle.grad_ncc(fixed, ref)
    np.testing.assert_allclose(sims, ref_sims, atol=1e-5, rtol=0)
    np.testing.assert_array_equal(obj, sims)
    # SimpleRayCasterWrapperFn in the C++ header: pose F P F^-1 R
    wrap = np.fromfile(tmp_path / "wrap.f32", np.float32).reshape(rows, cols)
    ref_w = oracle.drr_f32(vol.voxels, oracle_geom(vol), oracle_cams([cam]),
                           (F @ poses[0] @ np.linalg.inv(F) @ R)[None], step=step)[0]
    np.testing.assert_allclose(wrap, ref_w, rtol=1e-4, atol=1e-5)
    back = np.fromfile(tmp_path / "pose_back.f64", np.float64).reshape(4, 4)
    want = poses[1].astype(np.float32).astype(np.float64)
    want[3] = [0, 0, 0, 1]
    np.testing.assert_array_equal(back, want)
    # RunLevel and the same CMA-ES level stepped through JobSet::regi_step agree exactly
    lv = np.fromfile(tmp_path / "levels.f64", np.float64)
    np.testing.assert_array_equal(lv[:16], lv[16:32])
    assert lv[32] == lv[33] and lv[34] == lv[35] and lv[36] == lv[37] != 0
    psims = np.fromfile(tmp_path / "psims.f32", np.float32)
    ref_p = oracle.patch_ncc_ex(fixed, drr, radius=3, stride=2, mask=mask, use_mov_var_wgts=1)
    np.testing.assert_allclose(psims, ref_p, atol=1e-5, rtol=2e-6)
