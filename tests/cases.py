"""Named problem cases of the tests and of the kernel profiles, as one-call
solves.  `python tests/cases.py <case> [n]` solves each problem of the case
once and prints its iteration counts; the profiling commands run it under ncu.

  l2block   3D elasticity HDG k=2 and 3D Darcy HDG k=3 on n^3 cells, float-float
            block elimination (the two-field L2-panel kernel), PCG to 1e-10
  elasticity  3D elasticity HDG k=2 on n^3 cells, float-float path
  darcy-k3  3D Darcy HDG k=3 on n^3 cells, float-float path
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "gridaphybrid.jl_gb300"))

from gridaphybrid_gb300 import _lib  # noqa: E402
from gridaphybrid_gb300.operators import (CartesianDiscreteModel, DarcyHDG, ElasticityHDG,  # noqa: E402
                                          HybridAffineFEOperator, darcy_spaces, elasticity_spaces, solve)


def elasticity(n, k=2, precision=_lib.HDG_PREC_FF_BLOCK, seed=0, context=None):
    """3D elasticity HDG, E = 1, nu ~ U(0.2, 0.45) per cell, u = (sin pi x, cos pi y, xyz)."""
    nu = np.random.default_rng(seed).uniform(0.2, 0.45, size=n ** 3)
    model = CartesianDiscreteModel((0, 1) * 3, (n,) * 3)
    X, Y = elasticity_spaces(model, k)
    return HybridAffineFEOperator(ElasticityHDG(nu=nu, problem="smooth"), X, Y, [1, 2], [3],
                                  precision=precision, context=context)


def darcy(n, k=3, precision=_lib.HDG_PREC_FF_BLOCK, seed=1, context=None):
    """3D Darcy HDG, tau = 1, kappa = exp(N(0, 1)) per cell, p = prod sin(pi x_d)."""
    kap = np.exp(np.random.default_rng(seed).normal(size=n ** 3))
    model = CartesianDiscreteModel((0, 1) * 3, (n,) * 3)
    X, Y = darcy_spaces(model, k)
    return HybridAffineFEOperator(DarcyHDG(tau=1.0, problem="sin", kappa=kap), X, Y, [1, 2], [3],
                                  precision=precision, context=context)


CASES = {
    "l2block": lambda n: [elasticity(n, 2), darcy(n, 3)],
    "elasticity": lambda n: [elasticity(n, 2)],
    "darcy-k3": lambda n: [darcy(n, 3)],
}


def main(argv):
    if not argv or argv[0] not in CASES:
        print(__doc__)
        return 2
    n = int(argv[1]) if len(argv) > 1 else 8
    for op in CASES[argv[0]](n):
        xh = solve(op, solver="pcg", rtol=1e-10)
        print("%s n=%d: %d PCG iterations" % (argv[0], n, xh.iterations))
        op.pb.close()
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
