"""Algorithmic floating-point work per phase-space evaluation of the bench workload (the
rotating NFW model, 80 x 40 grid, l <= 12, 22^3 tanh-sinh nodes), from the oracle with every
operation tallied (orc_flops.cpp): the reference's algorithm in FP64, one evaluation = one
(grid point, velocity node) pair, bound or not.  Test infrastructure: the figures it prints
are the work unit of the bench's roofline.

    python oracle/count_flops.py [npoints]

FLOPs = add + mul + div + sqrt + TRANS_WEIGHT x trans (calls of exp, log10, pow, trig and
hyperbolic functions and their inverses), on a spread of grid points in the guess potential
(the radial integrals taken cumulatively, as the chosen form's loop does)."""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:] = [os.path.dirname(HERE)] + [p for p in sys.path if os.path.abspath(p) != HERE]
from oracle import oracle as O  # noqa: E402

TRANS_WEIGHT = 20


def main():
    import fjmodels_gb300 as F
    npoints = int(sys.argv[1]) if len(sys.argv) > 1 else 24
    nr, ng, npl = 80, 40, 7
    ar = O.log_grid(1e-3, 300.0, nr)
    rhl = O.guess_rhl(ar, ng, npl, "NFW")
    phil, Pr, Pr2 = O.compute_phil(ar, rhl, cumulative=True)
    x, w = F.tanh_sinh_rule(22)
    m = O.Model(ar, phil, Pr, Pr2, np.zeros(30), np.zeros(30), ng, alpha=1.667, beta=3.0, chi=1.0, k=0.5,
                xq=x, wq=w)
    E, D, _ = m.tabulate_delta(30)
    m.Egrid, m.Dgrid = E, D
    pts = np.linspace(0, nr * ng - 1, npoints).astype(int)
    _, c = O.flop_counts(m, pts)
    evals = len(pts) * len(x) ** 3
    per = {k: v / evals for k, v in c.items()}
    flops = per["add"] + per["mul"] + per["div"] + per["sqrt"] + TRANS_WEIGHT * per["trans"]
    print(json.dumps({"workload": "NFW 80x40, l<=12, 22^3 tanh-sinh nodes, guess potential",
                      "points": len(pts), "evaluations": evals, "per_evaluation": per,
                      "trans_weight": TRANS_WEIGHT, "flops_per_evaluation": flops}, indent=1))


if __name__ == "__main__":
    main()
