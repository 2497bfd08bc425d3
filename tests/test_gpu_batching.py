"""GPU tests of size-class batching (hdg_batch_*): the persistent fused
integrate -> condense launches give the same assembled skeleton systems and
solutions as assembling each problem on its own (the same per-output
arithmetic, whatever tile the autotuner picks), graph replays follow new
permeability fields, and the tuner reports a tile per class."""
import ctypes

import numpy as np
import pytest

import gridaphybrid_gb300 as gh
from gridaphybrid_gb300 import _lib
from gridaphybrid_gb300.batching import Batch, batching_workload

pytestmark = pytest.mark.gpu

SPECS = [(2, 9, 1), (2, 7, 3), (3, 3, 2), (2, 12, 2), (2, 6, 1), (3, 4, 1), (2, 5, 3), (3, 3, 2)]


def _specs(seed=0):
    rng = np.random.default_rng(seed)
    return [{"D": D, "n": n, "k": k, "kappa": np.exp(1.5 * rng.normal(size=n ** D))} for D, n, k in SPECS]


def _single(spec, precision):
    D, n, k = spec["D"], spec["n"], spec["k"]
    model = gh.CartesianDiscreteModel((0, 1) * D, (n,) * D)
    X, Y = gh.darcy_spaces(model, k)
    op = gh.HybridAffineFEOperator(gh.DarcyHDG(tau=1.0, problem="sin", kappa=spec["kappa"]), X, Y, [1, 2], [3],
                                   precision=precision)
    _, _, val, rhs = op.skeleton_system()
    xh = gh.solve(op, solver="pcg", rtol=1e-10)
    return val, rhs, xh.free_dof_values.copy()


@pytest.mark.parametrize("precision", [_lib.HDG_PREC_FF_BLOCK, _lib.HDG_PREC_FP64])
def test_batch_equals_single_problem_assembly(precision):
    specs = _specs()
    with Batch(specs) as b:
        bad = b.assemble(precision)
        assert (bad == 0).all()
        its, rel = b.solve(rtol=1e-10)
        assert (rel <= 1e-10).all()
        for i, spec in enumerate(specs):
            val, rhs, sol = _single(spec, precision)
            bval, brhs = b.skeleton_values(i)
            assert np.array_equal(bval, val) and np.array_equal(brhs, rhs)
            assert np.array_equal(b.free_dof_values(i), sol)
        tun = b.tuning(precision)
    assert {(t["D"], t["k"]) for t in tun} == {(D, k) for D, _, k in SPECS}
    assert all(t["threads_per_cell"] in (32, 64, 128, 256) for t in tun)
    assert sum(t["cells"] for t in tun) == sum(n ** D for D, n, _ in SPECS)


def test_graph_replay_follows_new_permeability():
    specs = _specs(1)
    with Batch(specs) as b:
        b.assemble(_lib.HDG_PREC_FF_BLOCK)   # tunes, captures the graph
        b.assemble(_lib.HDG_PREC_FF_BLOCK)   # replays it
        new = np.exp(np.random.default_rng(9).normal(size=specs[3]["n"] ** 2))
        c = b.ctx
        c.check(c.lib.hdg_set_permeability(b.pbs[3].h, _lib.ptr(new)))
        b.assemble(_lib.HDG_PREC_FF_BLOCK)   # replay with the new field
        bval, brhs = b.skeleton_values(3)
    spec = dict(specs[3])
    spec["kappa"] = new
    val, rhs, _ = _single(spec, _lib.HDG_PREC_FF_BLOCK)
    assert np.array_equal(bval, val) and np.array_equal(brhs, rhs)


def test_batch_rejects_foreign_problems_and_precisions():
    lib = _lib.load()
    other = gh.Context(0)
    specs = _specs(2)[:2]
    with Batch(specs) as b:
        model = gh.CartesianDiscreteModel((0, 1, 0, 1), (4, 4))
        from gridaphybrid_gb300.operators import _Problem
        foreign = _Problem(other, model, 1)
        handles = (ctypes.c_void_p * 2)(b.pbs[0].h.value, foreign.h.value)
        h = ctypes.c_void_p()
        assert lib.hdg_batch_create(b.ctx.handle, 2, handles, ctypes.byref(h)) == _lib.HDG_ERR_INVALID
        with pytest.raises(_lib.HdgError):
            b.assemble(_lib.HDG_PREC_FP32_REFINED)
        foreign.close()
    other.close()
