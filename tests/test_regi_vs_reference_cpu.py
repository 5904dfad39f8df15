"""The library's CMA-ES against xReg's own optimizer on the same registration
objective.

tests/golden/regi_reference_runs.json records runs of the reference's vendored
cmaes.c (compiled from the xReg sources; make_regi_golden.py) driving a
single-view registration level (tests/golden/regi_problem.py: the oracle's CPU
DRR + grad-NCC, pose offsets about the volume centre, as
Intensity2D3DRegiCMAES::run drives it).  The library's CMA-ES runs the same
level from the same start with the same lambda, step sizes and stop rules.
The random streams differ, so the comparison is of outcomes: both end within
the registration tolerance of the truth (0.05 deg / 0.1 mm), at each other's
best value to within 1e-6, at poses within that tolerance of each other, in
generation counts within 2x of the reference's."""
import json
from pathlib import Path

import numpy as np


def test_level_reaches_what_the_reference_optimizer_reaches(xr):
    from oracle import oracle as O
    from tests.golden import regi_problem as RP
    from xreg_gb300.cmaes import CMAES
    d = json.loads((Path(__file__).parent / "golden" / "regi_reference_runs.json").read_text())
    assert d["lambda"] == RP.LAM and d["sigma"] == RP.SIGMA.tolist() and d["max_iter"] == RP.MAX_ITER
    O.set_threads(0)
    P = RP.Problem()
    ours_gens, ref_gens = [], []
    for run in d["runs"]:
        es = CMAES(np.zeros(6), RP.SIGMA, RP.LAM, seed=run["seed"])
        es.set_stop(tol_fun=RP.TOL_FUN, tol_x=RP.TOL_X, max_iter=RP.MAX_ITER)
        while es.test_for_termination() is None:
            pop = es.sample_population()
            es.update_distribution(P.values(pop))
        st = es.state()
        x_ref = np.array(run["best_x"])
        rot, trans = P.error(st["best_x"])
        assert rot <= 0.05 and trans <= 0.1, (run["seed"], rot, trans)
        assert run["error_deg"] <= 0.05 and run["error_mm"] <= 0.1
        assert abs(st["best_f"] - run["best_f"]) <= 1e-6, (st["best_f"], run["best_f"])
        rot_ab, trans_ab = P.error(st["best_x"], P.poses(x_ref)[0])
        assert rot_ab <= 0.05 and trans_ab <= 0.1, (rot_ab, trans_ab)
        ours_gens.append(st["generation"])
        ref_gens.append(run["generations"])
    ratio = np.mean(ours_gens) / np.mean(ref_gens)
    assert 0.5 < ratio < 2.0, (ours_gens, ref_gens)
