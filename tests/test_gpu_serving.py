"""GPU tests of the native serving loop (hdg_server_*): a result is the same
alone and in a mix of concurrent requests, admission respects the HBM
budget, resident meshes are reused, unsupported shapes are rejected at
submit, and the footprint bound covers what a solve reserves."""
import ctypes

import numpy as np
import pytest

import gridaphybrid_gb300 as gh
from gridaphybrid_gb300 import _lib
from gridaphybrid_gb300.serving import Server, kappa_for

pytestmark = pytest.mark.gpu

# A result must not depend on the mix: the kernels reduce in a fixed order and
# the grid of every launch depends only on the request, so the bits are equal.
RTOL_MIX = 0.0


def _solve_direct_api(D, n, k, kappa, precision):
    model = gh.CartesianDiscreteModel((0, 1) * D, (n,) * D)
    X, Y = gh.darcy_spaces(model, k)
    op = gh.HybridAffineFEOperator(gh.DarcyHDG(tau=1.0, problem="sin", kappa=kappa), X, Y, [1, 2], [3],
                                   precision=precision)
    xh = gh.solve(op, solver="pcg", rtol=1e-10)
    return xh.free_dof_values.copy()


@pytest.mark.parametrize("precision", [_lib.HDG_PREC_FF_BLOCK, _lib.HDG_PREC_FP64])
def test_same_result_alone_and_in_the_mix(precision):
    target = (3, 6, 2)
    kap = kappa_for(3, 6, 11)
    with Server(slots=4) as srv:
        t = srv.submit(*target, kappa=kap, precision=precision, want_solution=True)
        srv.drain()
        alone = {r["ticket"]: r for r in srv.poll(max_items=16)}[t]
        assert alone["status"] == 0
        mix = [(2, 40, 1), (2, 24, 3), (3, 8, 1), (3, 6, 2), (2, 64, 2), (3, 10, 2), (2, 16, 1)]
        tickets = []
        for i, (D, n, k) in enumerate(mix):
            tickets.append(srv.submit(D, n, k, kappa=kappa_for(D, n, 100 + i), precision=precision,
                                      want_solution=True))
            if i == 3:
                tt = srv.submit(*target, kappa=kap, precision=precision, want_solution=True)
        srv.drain()
        res = {r["ticket"]: r for r in srv.poll(max_items=64)}
        st = srv.stats()
    assert all(res[x]["status"] == 0 for x in tickets + [tt])
    assert st["max_concurrent"] >= 2  # the mix overlapped on the device
    inmix = res[tt]["solution"]
    assert np.abs(inmix - alone["solution"]).max() <= RTOL_MIX * np.abs(alone["solution"]).max()
    # and the same as the single-problem API
    ref = _solve_direct_api(3, 6, 2, kap, precision)
    assert np.array_equal(ref, alone["solution"])
    assert alone["err_flux"] == res[tt]["err_flux"]


def test_admission_respects_budget_and_reuses_meshes():
    """Budget for one (3, 10, 2) request: its resident mesh is reused by the next
    request of that shape and evicted to admit a different one."""
    def fp(D, n, k):
        b = ctypes.c_double()
        assert _lib.load().hdg_footprint(D, n, k, _lib.HDG_PREC_FF_BLOCK, _lib.HDG_SOLVER_PCG, ctypes.byref(b)) == 0
        return b.value

    shapes = [(3, 10, 2), (3, 10, 2), (3, 12, 1), (3, 10, 2)]
    budget = 1.02 * fp(3, 10, 2)
    assert fp(3, 12, 1) < budget
    with Server(slots=1, budget_bytes=budget) as srv:
        for i, (D, n, k) in enumerate(shapes):  # one at a time: the admission order is the submission order
            srv.submit(D, n, k, kappa=kappa_for(D, n, i), precision=_lib.HDG_PREC_FF_BLOCK)
            srv.drain()
        res = sorted(srv.poll(max_items=16), key=lambda r: r["ticket"])
        st = srv.stats()
    assert len(res) == len(shapes) and all(r["status"] == 0 for r in res)
    assert [r["reused_mesh"] for r in res] == [0, 1, 0, 0]
    assert st["peak_bytes"] <= budget
    assert st["mesh_hits"] >= 1 and st["evictions"] >= 1


def test_requests_overlap_under_a_budget():
    """Eight slots, a budget for about three of the requests at a time: the
    requests run concurrently and the reserved bytes never exceed the budget."""
    b = ctypes.c_double()
    assert _lib.load().hdg_footprint(2, 40, 1, _lib.HDG_PREC_FF_BLOCK, _lib.HDG_SOLVER_PCG, ctypes.byref(b)) == 0
    budget = 3.2 * b.value
    with Server(slots=8, budget_bytes=budget) as srv:
        for i in range(12):
            srv.submit(2, 40 + (i % 4), 1, kappa=kappa_for(2, 40 + (i % 4), i), precision=_lib.HDG_PREC_FF_BLOCK)
        srv.drain()
        res = srv.poll(max_items=16)
        st = srv.stats()
    assert len(res) == 12 and all(r["status"] == 0 for r in res)
    assert 2 <= st["max_concurrent"] <= 3
    assert st["peak_bytes"] <= budget


def test_shortest_work_first_admission():
    """With the slot busy, queued small requests are admitted before a queued
    large one that arrived earlier (none has waited long enough to age)."""
    with Server(slots=1) as srv:
        srv.submit(3, 16, 2, kappa=kappa_for(3, 16, 0))  # occupies the slot
        big = srv.submit(3, 16, 2, kappa=kappa_for(3, 16, 1))
        small = [srv.submit(2, 8, 1, kappa=kappa_for(2, 8, 2 + i)) for i in range(3)]
        srv.drain()
        order = [r["ticket"] for r in srv.poll(max_items=8)]
    assert len(order) == 5
    assert order.index(big) > max(order.index(t) for t in small)


def test_mesh_reuse_gives_the_fresh_result():
    with Server(slots=1) as srv:
        a = srv.submit(2, 20, 2, kappa=kappa_for(2, 20, 1), want_solution=True)
        b = srv.submit(2, 20, 2, kappa=kappa_for(2, 20, 2), want_solution=True)
        c = srv.submit(2, 20, 2, kappa=kappa_for(2, 20, 1), want_solution=True)
        srv.drain()
        res = {r["ticket"]: r for r in srv.poll(max_items=8)}
    assert res[a]["reused_mesh"] == 0 and res[b]["reused_mesh"] == 1 and res[c]["reused_mesh"] == 1
    assert np.array_equal(res[a]["solution"], res[c]["solution"])
    assert not np.array_equal(res[a]["solution"], res[b]["solution"])


def test_unsupported_shape_rejected_at_submit():
    with Server(slots=1) as srv:
        with pytest.raises(_lib.HdgError):
            srv.submit(3, 4, 4, precision=_lib.HDG_PREC_FF_BLOCK)
        with pytest.raises(_lib.HdgError):
            srv.submit(3, 4, 3, precision=_lib.HDG_PREC_FP32_REFINED)
        with pytest.raises(_lib.HdgError):
            srv.submit(2, 0, 1)


@pytest.mark.parametrize("precision", [_lib.HDG_PREC_FF_BLOCK, _lib.HDG_PREC_FP64])
def test_3d_k3_request_served(precision):
    """3D k=3 (cell block n = 352, condensed by the L2-panel block
    elimination) through the serving loop: the single-problem API's bits."""
    kap = kappa_for(3, 4, 5)
    with Server(slots=2) as srv:
        t = srv.submit(3, 4, 3, kappa=kap, precision=precision, want_solution=True)
        srv.drain()
        res = {r["ticket"]: r for r in srv.poll(max_items=4)}
    assert res[t]["status"] == 0
    assert np.array_equal(res[t]["solution"], _solve_direct_api(3, 4, 3, kap, precision))


def test_footprint_bounds_the_reserved_bytes():
    lib = _lib.load()
    for (D, n, k, prec) in [(2, 32, 1, _lib.HDG_PREC_FP64), (2, 24, 3, _lib.HDG_PREC_FF_BLOCK),
                            (3, 8, 2, _lib.HDG_PREC_FF_BLOCK), (3, 8, 2, _lib.HDG_PREC_FP64),
                            (3, 6, 1, _lib.HDG_PREC_FP32_REFINED), (3, 5, 3, _lib.HDG_PREC_FF_BLOCK),
                            (3, 5, 3, _lib.HDG_PREC_FP64)]:
        model = gh.CartesianDiscreteModel((0, 1) * D, (n,) * D)
        X, Y = gh.darcy_spaces(model, k)
        op = gh.HybridAffineFEOperator(gh.DarcyHDG(tau=1.0, problem="sin"), X, Y, [1, 2], [3], precision=prec)
        xh = gh.solve(op, solver="pcg", rtol=1e-10)
        xh.l2_errors()
        used, bound = ctypes.c_double(), ctypes.c_double()
        assert lib.hdg_problem_device_bytes(op.pb.h, ctypes.byref(used)) == 0
        assert lib.hdg_footprint(D, n, k, prec, _lib.HDG_SOLVER_PCG, ctypes.byref(bound)) == 0
        assert 0 < used.value <= bound.value
