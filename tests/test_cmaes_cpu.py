"""The library's CMA-ES against the reference's own vendored cmaes.c (compiled
from the xReg sources into oracle/_ref when they are present).  Both are driven
the way Intensity2D3DRegiCMAES::run drives cmaes.c; the random streams differ,
so the comparison is behavioural: both reach the optimum of standard test
functions to the same accuracy in a comparable number of generations."""
import numpy as np
import pytest


def sphere(x):
    return float(np.sum(x * x))


def ellipsoid(x):
    n = x.size
    return float(np.sum((1e3 ** (np.arange(n) / (n - 1))) * x * x))


def rosenbrock(x):
    return float(np.sum(100.0 * (x[1:] - x[:-1] ** 2) ** 2 + (1 - x[:-1]) ** 2))


def _run_ours(f, x0, sd, lam, seed, tol_fun, max_iter=5000):
    from xreg_gb300.cmaes import CMAES
    es = CMAES(x0, sd, lam, seed)
    es.set_stop(tol_fun=tol_fun, tol_x=1e-12, max_iter=max_iter)
    while es.test_for_termination() is None:
        pop = es.sample_population()
        es.update_distribution([f(p) for p in pop])
    st = es.state()
    return st["mean"], st["generation"]


def _run_ref(f, x0, sd, lam, seed, tol_fun, max_iter=5000):
    from oracle import oracle as O
    try:
        es = O.RefCMAES(x0, sd, lam, seed, tol_fun=tol_fun, tol_x=1e-12, max_iter=max_iter)
    except FileNotFoundError:
        pytest.skip("reference CMA-ES sources not available")
    while not es.stop():
        pop = es.sample()
        es.update([f(p) for p in pop])
    return es.mean(), es.generation()


@pytest.mark.parametrize("fn,opt,tolx", [(sphere, 0.0, 1e-6), (ellipsoid, 0.0, 1e-5), (rosenbrock, 1.0, 1e-4)])
def test_converges_like_reference(xr, fn, opt, tolx):
    n, lam = 6, 20
    x0 = np.full(n, 0.5 if fn is rosenbrock else 3.0)
    sd = np.full(n, 1.0)
    gens_ours, gens_ref = [], []
    for seed in (1, 2, 3):
        m1, g1 = _run_ours(fn, x0, sd, lam, seed, 1e-14)
        m2, g2 = _run_ref(fn, x0, sd, lam, seed, 1e-14)
        assert np.max(np.abs(m1 - opt)) < tolx, (fn.__name__, m1)
        assert np.max(np.abs(m2 - opt)) < tolx, (fn.__name__, m2)
        gens_ours.append(g1)
        gens_ref.append(g2)
    r = np.mean(gens_ours) / np.mean(gens_ref)
    assert 0.5 < r < 2.0, (gens_ours, gens_ref)


def test_against_reference_golden_runs(xr):
    """The same comparison against committed runs of the reference's cmaes.c
    (tests/golden/cmaes_reference_runs.json, made by make_cmaes_golden.py), so it
    also holds where the xReg sources are absent: every run of ours reaches the
    optimum the reference reached, in a comparable number of generations."""
    import json
    from pathlib import Path
    d = json.loads((Path(__file__).parent / "golden" / "cmaes_reference_runs.json").read_text())
    fns = {"sphere": (sphere, 0.0, 1e-6), "ellipsoid": (ellipsoid, 0.0, 1e-5), "rosenbrock": (rosenbrock, 1.0, 1e-4)}
    for name, (fn, opt, tolx) in fns.items():
        runs = [r for r in d["runs"] if r["function"] == name]
        assert len(runs) == 3
        ours = []
        for r in runs:
            assert np.max(np.abs(np.array(r["final_mean"]) - opt)) < tolx
            m, g = _run_ours(fn, np.array(r["x0"]), np.full(r["dim"], 1.0), r["lambda"], r["seed"], 1e-14)
            assert np.max(np.abs(m - opt)) < tolx, (name, m)
            ours.append(g)
        ratio = np.mean(ours) / np.mean([r["generations"] for r in runs])
        assert 0.5 < ratio < 2.0, (name, ours, [r["generations"] for r in runs])


def test_registration_like_objective(xr):
    """6 parameters with xReg's per-coordinate scales (radians vs mm) and bounds."""
    target = np.array([0.05, -0.03, 0.08, 4.0, -6.0, 9.0])
    scale = np.array([0.1, 0.1, 0.1, 10.0, 10.0, 10.0])
    f = lambda x: float(np.sum(((x - target) / scale) ** 2))
    from xreg_gb300.cmaes import CMAES
    es = CMAES(np.zeros(6), [0.15, 0.15, 0.15, 20.0, 20.0, 20.0], 30, 7)
    es.set_stop(tol_fun=1e-12, tol_x=1e-9, max_iter=400)
    bounds = [0.5, 0.5, 0.5, 50.0, 50.0, 50.0]
    while es.test_for_termination() is None:
        pop = es.sample_within_bounds(bounds)
        assert np.all(np.abs(pop) <= np.array(bounds))
        es.update_distribution([f(p) for p in pop])
    np.testing.assert_allclose(es.state()["mean"], target, atol=1e-4)


def test_reproducible_and_validated(xr):
    from xreg_gb300 import _lib
    from xreg_gb300.cmaes import CMAES
    a = CMAES(np.ones(4), np.ones(4), 8, 42).sample_population().copy()
    b = CMAES(np.ones(4), np.ones(4), 8, 42).sample_population().copy()
    np.testing.assert_array_equal(a, b)
    with pytest.raises(_lib.XRegError):
        CMAES(np.ones(3), np.array([1.0, 0.0, 1.0]), 8)
    with pytest.raises(_lib.XRegError):
        CMAES(np.ones(3), np.ones(3), 1)


def _run_dfo(f, x0, lo, hi, rho_beg, rho_end, max_iter=500):
    from xreg_gb300.cmaes import TrustRegionDFO
    d = TrustRegionDFO(x0, lo, hi, rho_beg, rho_end, max_iter)
    n_eval = 0
    while d.test_for_termination() is None:
        pts = d.ask()
        assert np.all(pts >= lo - 1e-12) and np.all(pts <= hi + 1e-12)
        d.tell([f(p) for p in pts])
        n_eval += len(pts)
    return d.state(), n_eval


def test_trust_region_dfo_on_quadratics_and_rosenbrock(xr):
    scale = np.array([0.1, 0.1, 0.1, 10.0, 10.0, 10.0])
    target = np.array([0.02, -0.03, 0.01, 2.0, -3.0, 4.0])
    lo, hi = -2.5 * scale, 2.5 * scale
    f = lambda x: float(np.sum(((x - target) / scale) ** 2) + 0.3 * ((x[0] - target[0]) / scale[0]) *
                        ((x[4] - target[4]) / scale[4]))
    st, ne = _run_dfo(f, np.zeros(6), lo, hi, 0.2, 1e-6)
    np.testing.assert_allclose(st["best_x"], target, atol=1e-4 * 10)
    assert st["best_f"] < f(np.zeros(6)) * 1e-6
    # a bound-active optimum: the solution sits on the box
    g = lambda x: float(np.sum((x - 3.0) ** 2))
    st2, _ = _run_dfo(g, np.zeros(3), -np.ones(3), np.ones(3), 0.5, 1e-7)
    np.testing.assert_allclose(st2["best_x"], np.ones(3), atol=1e-9)
    # Rosenbrock in 4-D from a bounded start
    st3, _ = _run_dfo(rosenbrock, np.full(4, -0.5), -2 * np.ones(4), 2 * np.ones(4), 0.5, 1e-9, max_iter=4000)
    assert st3["best_f"] < 1e-3, st3


def test_regi_pose_map(xr):
    """xr_regi_pose_map: C @ Exp(x) @ inv(C) @ start for each row, against the
    same composition in numpy (host code only)."""
    from xreg_gb300 import api
    from xreg_gb300.se3 import exp_se3_batch
    rng = np.random.default_rng(5)
    C = exp_se3_batch(np.concatenate([rng.normal(0, 0.3, 3), rng.normal(0, 50, 3)])[None])[0]
    start = exp_se3_batch(np.concatenate([rng.normal(0, 0.3, 3), rng.normal(0, 200, 3)])[None])[0]
    xs = np.concatenate([rng.normal(0, 0.1, (9, 3)), rng.normal(0, 10, (9, 3))], axis=1)
    got = api.regi_pose_map(C, start, xs)
    want = np.einsum("ij,njk,kl->nil", C, exp_se3_batch(xs), np.linalg.inv(C) @ start)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-9)
    assert api.regi_pose_map(C, start, np.zeros((0, 6))).shape == (0, 4, 4)
