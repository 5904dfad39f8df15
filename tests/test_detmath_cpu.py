"""The optimizer's own transcendental functions and random normals
(xr_cmaes_core.h), compiled for the host exactly as the library is
(-ffp-contract=off), against numpy: ln, exp and sin/cos within a few ulp over
the ranges the optimizer uses them on, Box-Muller normals with the moments and
distribution of N(0, 1), independent streams per (generation, candidate,
draw), and the level's pose map C Exp(x) C^-1 start against the same
composition in numpy.  The device runs the same source (bit equality with the
host is checked on the GPU, tests/test_gpu_cmaes_device.py)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = tmp_path_factory.mktemp("detmath") / "detmath_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", f"-I{ROOT / 'xreg_gb300' / 'csrc'}",
                    f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp/detmath_check.cpp"), "-o", str(out)], check=True)
    return out


def _run(exe, mode, x, tmp_path):
    fi, fo = tmp_path / "in.f64", tmp_path / "out.f64"
    np.ascontiguousarray(x, dtype=np.float64).tofile(fi)
    subprocess.run([str(exe), mode, str(fi), str(fo)], check=True)
    return np.fromfile(fo, dtype=np.float64)


def _ulp_err(got, want):
    return np.max(np.abs(got - want) / np.spacing(np.abs(want)))


def test_ln(exe, tmp_path):
    rng = np.random.default_rng(1)
    u = np.concatenate([(np.arange(1, 20001) * 2.0 ** -53) * 2 ** 38, rng.random(50000) + 2.0 ** -53,
                        np.exp(rng.uniform(-700, 700, 20000)), [1.0, 0.5, 2.0, np.sqrt(0.5), 5e-324 * 2 ** 60]])
    got = _run(exe, "ln", u, tmp_path)
    want = np.log(u)
    nz = want != 0
    assert _ulp_err(got[nz], want[nz]) <= 2.0
    assert got[np.flatnonzero(u == 1.0)[0]] == 0.0


def test_exp(exe, tmp_path):
    rng = np.random.default_rng(2)
    y = np.concatenate([rng.uniform(-700, 700, 20000), rng.uniform(-2, 2, 20000), [0.0, -1e-300, 1e-20]])
    got = _run(exe, "exp", y, tmp_path)
    assert _ulp_err(got, np.exp(y)) <= 2.0
    edge = _run(exe, "exp", np.array([800.0, -800.0]), tmp_path)
    assert np.isinf(edge[0]) and edge[1] == 0.0


def test_sincos(exe, tmp_path):
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-8, 8, 40000), rng.uniform(0, 2 * np.pi, 20000), rng.uniform(-1e-6, 1e-6, 2000),
                        np.arange(-16, 17) * (np.pi / 4)])
    got = _run(exe, "sincos", x, tmp_path).reshape(-1, 2)
    # absolute error relative to 1 (the result's scale near its zeros)
    assert np.max(np.abs(got[:, 0] - np.sin(x))) <= 4e-16
    assert np.max(np.abs(got[:, 1] - np.cos(x))) <= 4e-16
    small = (np.abs(x) < 1e-6) & (x != 0)
    assert _ulp_err(got[small, 0], np.sin(x[small])) <= 1.0  # relative accuracy near 0


def test_normals(exe, tmp_path):
    # 100000 pairs: generation, candidate, draw and pair counters all varied
    n = 100000
    rng = np.random.default_rng(4)
    rows = np.stack([np.full(n, 7.0), rng.integers(0, 300, n), rng.integers(0, 100, n), rng.integers(0, 5, n),
                     rng.integers(0, 3, n)], axis=1)
    z = _run(exe, "normals", rows, tmp_path)
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
    assert abs(np.mean(z ** 3)) < 0.03 and abs(np.mean(z ** 4) - 3.0) < 0.06
    from scipy import stats
    assert stats.kstest(z, "norm").pvalue > 1e-3
    # a redraw (next attempt) or another candidate gives another stream; the same counters the same bits
    a = _run(exe, "normals", np.array([[3, 1, 2, 0, 0], [3, 1, 2, 1, 0], [3, 1, 3, 0, 0], [3, 2, 2, 0, 0],
                                       [3, 1, 2, 0, 0]], dtype=np.float64), tmp_path).reshape(-1, 2)
    assert len({tuple(r) for r in a[:4]}) == 4
    np.testing.assert_array_equal(a[0], a[4])


def test_pose_map(exe, tmp_path):
    from xreg_gb300.se3 import exp_se3_batch
    rng = np.random.default_rng(5)
    C = exp_se3_batch(np.concatenate([rng.normal(0, 0.3, 3), rng.normal(0, 50, 3)])[None])[0]
    start = exp_se3_batch(np.concatenate([rng.normal(0, 0.3, 3), rng.normal(0, 200, 3)])[None])[0]
    B = np.linalg.inv(C) @ start
    xs = np.concatenate([rng.normal(0, 0.2, (50, 3)), rng.normal(0, 10, (50, 3))], axis=1)
    xs[0] = 0.0
    xs[1, :3] = 1e-15
    got = _run(exe, "posemap", np.concatenate([C.ravel(), B.ravel(), xs.ravel()]), tmp_path).reshape(-1, 4, 4)
    want = np.einsum("ij,njk,kl->nil", C, exp_se3_batch(xs), B)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-10)
