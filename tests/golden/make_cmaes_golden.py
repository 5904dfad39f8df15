"""Generates cmaes_reference_runs.json: runs of the reference's own vendored
CMA-ES (xReg third_party/cmaes/cmaes.c, compiled from the xReg sources into
oracle/_ref by oracle/Makefile) on the standard test functions the CMA-ES tests
use, driven as Intensity2D3DRegiCMAES::run drives it (sample, evaluate, update,
test for termination).  Run from the repository root where the xReg sources
are present:  python tests/golden/make_cmaes_golden.py [xreg source dir]"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402

FUNCS = {
    "sphere": lambda x: float(np.sum(x * x)),
    "ellipsoid": lambda x: float(np.sum((1e3 ** (np.arange(x.size) / (x.size - 1))) * x * x)),
    "rosenbrock": lambda x: float(np.sum(100.0 * (x[1:] - x[:-1] ** 2) ** 2 + (1 - x[:-1]) ** 2)),
}


def main():
    if len(sys.argv) > 1:
        O.build_ref(sys.argv[1])
    elif O.build_ref() is None:
        sys.exit("the reference CMA-ES sources are not available")
    runs = []
    n, lam = 6, 20
    for name, f in FUNCS.items():
        x0 = np.full(n, 0.5 if name == "rosenbrock" else 3.0)
        for seed in (1, 2, 3):
            es = O.RefCMAES(x0, np.full(n, 1.0), lam, seed, tol_fun=1e-14, tol_x=1e-12, max_iter=5000)
            first = None
            while not es.stop():
                pop = es.sample()
                if first is None:
                    first = pop.copy()
                es.update([f(p) for p in pop])
            runs.append({"function": name, "seed": seed, "dim": n, "lambda": lam, "x0": x0.tolist(),
                         "generations": es.generation(), "final_mean": es.mean().tolist(),
                         "first_population": first.tolist()})
    out = Path(__file__).with_name("cmaes_reference_runs.json")
    out.write_text(json.dumps({"source": "xReg third_party/cmaes/cmaes.c (cmaes_init with these "
                                         "parameters, tol_fun 1e-14, tol_x 1e-12, max_iter 5000)",
                               "runs": runs}, indent=1))
    print(out)


if __name__ == "__main__":
    main()
