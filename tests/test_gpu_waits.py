"""The bounded device waits give up, say so, and leave the context usable.

The bulk-copy rings (skeleton SpMV, persistent PCG) wait on mbarriers and the
persistent PCG's grid barrier waits on a generation word; both waits are
bounded.  hdg_check_bounded_waits runs the same two wait primitives against
a barrier phase and a word that nothing completes or writes (nothing else is
in flight), with a short poll limit.  Each must report that it gave up, and
the same context must then still run a solve that matches the oracle.
"""
import numpy as np
import pytest

import gridaphybrid_gb300 as gh
from gridaphybrid_gb300 import _lib
from oracle import oracle

pytestmark = pytest.mark.gpu

BULK_WAIT_POLLS = 1 << 18
GRID_WAIT_POLLS = 1 << 22


def test_bounded_waits_expire_and_context_stays_usable():
    ctx = gh.default_context()
    expired = np.zeros(2, dtype=np.int32)
    ns = np.zeros(2)
    ctx.check(ctx.lib.hdg_check_bounded_waits(ctx.handle, 4096, _lib.ptr(expired), _lib.ptr(ns)))
    assert expired.tolist() == [1, 1]
    assert (ns > 0).all()
    limits_s = (ns[0] * BULK_WAIT_POLLS * 1e-9, ns[1] * GRID_WAIT_POLLS * 1e-9)
    print("ns per poll (mbarrier, grid word): %.1f %.1f; production limits %.2f s, %.2f s"
          % (ns[0], ns[1], *limits_s))
    # the production limits give up after about a second (3.8 us per mbarrier
    # poll and 0.2 us per generation-word poll measured on a GB300)
    assert max(limits_s) < 5.0
    # out-of-range poll counts are refused before any launch
    with pytest.raises(gh.HdgError):
        ctx.check(ctx.lib.hdg_check_bounded_waits(ctx.handle, 0, _lib.ptr(expired), _lib.ptr(ns)))

    model = gh.CartesianDiscreteModel((0, 1, 0, 1), (6, 6))
    X, Y = gh.darcy_spaces(model, 2)
    kappa = np.exp(np.random.default_rng(0).normal(size=36))
    op = gh.HybridAffineFEOperator(gh.DarcyHDG(tau=1.0, problem="sin", kappa=kappa), X, Y, [1, 2], [3],
                                   precision=_lib.HDG_PREC_FF_BLOCK, context=ctx)
    xh = gh.solve(op, solver="pcg", rtol=1e-12)
    ref = oracle.solve_darcy(2, 2, (6, 6), problem=oracle.PROBLEM_SIN, kappa=kappa, solver=0)
    assert np.abs(xh.skeleton - ref["lam"]).max() <= 1e-8 * np.abs(ref["lam"]).max()
    op.pb.close()
