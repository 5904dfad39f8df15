"""Generates regi_reference_runs.json: the reference's own vendored CMA-ES
(xReg third_party/cmaes/cmaes.c, compiled from the xReg sources into
oracle/_ref by oracle/Makefile) driving the registration level of
regi_problem.py on the oracle's CPU objective (DRR + grad-NCC), as
Intensity2D3DRegiCMAES::run drives it (sample, evaluate, update, test for
termination), from the same start, step sizes, lambda and stop rules the
library's test uses.  Run from the repository root where the xReg sources are
present:  XREG_REFERENCE_DIR=<xreg sources> python tests/golden/make_regi_golden.py"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from tests.golden import regi_problem as RP  # noqa: E402


def main():
    if O.build_ref() is None:
        sys.exit("the reference CMA-ES sources are not available (set XREG_REFERENCE_DIR)")
    O.set_threads(0)
    P = RP.Problem()
    runs = []
    for seed in RP.SEEDS:
        es = O.RefCMAES(np.zeros(6), RP.SIGMA, RP.LAM, seed, tol_fun=RP.TOL_FUN, tol_x=RP.TOL_X,
                        max_iter=RP.MAX_ITER)
        n_eval = 0
        best_f, best_x = np.inf, None
        while not es.stop():
            pop = es.sample().copy()
            f = P.values(pop)
            n_eval += len(pop)
            k = int(np.argmin(f))
            if f[k] < best_f:
                best_f, best_x = float(f[k]), pop[k].copy()
            es.update(f)
        mean = es.mean()
        rot, trans = P.error(best_x)
        runs.append({"seed": seed, "generations": int(es.generation()), "evaluations": n_eval, "best_f": best_f,
                     "best_x": best_x.tolist(), "final_mean": mean.tolist(), "error_deg": rot, "error_mm": trans})
        print(runs[-1])
    out = {"problem": "tests/golden/regi_problem.py", "optimizer": "xReg third_party/cmaes/cmaes.c",
           "lambda": RP.LAM, "sigma": RP.SIGMA.tolist(), "tol_fun": RP.TOL_FUN, "tol_x": RP.TOL_X,
           "max_iter": RP.MAX_ITER, "runs": runs}
    (Path(__file__).parent / "regi_reference_runs.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
