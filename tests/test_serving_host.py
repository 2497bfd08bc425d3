"""CPU checks of the serving workload generator and the footprint bound used
for HBM admission (no device calls)."""
import ctypes

import numpy as np

from gridaphybrid_gb300 import _lib
from gridaphybrid_gb300 import serving


def test_trace_is_seeded_and_in_range():
    a = serving.poisson_trace(rate=200.0, seconds=5.0, seed=3)
    b = serving.poisson_trace(rate=200.0, seconds=5.0, seed=3)
    assert a == b
    assert 800 < len(a) < 1200  # Poisson(1000)
    t = np.array([x[0] for x in a])
    assert np.all(np.diff(t) > 0) and t[-1] < 5.0
    for (_, D, n, k, _) in a:
        if D == 2:
            assert serving.N2D_RANGE[0] <= n <= serving.N2D_RANGE[1] and k in serving.K2D
        else:
            assert D == 3 and serving.N3D_RANGE[0] <= n <= serving.N3D_RANGE[1] and k in serving.K3D
    frac2d = np.mean([x[1] == 2 for x in a])
    assert abs(frac2d - serving.P_2D) < 0.05


def test_kappa_is_reproducible_lognormal():
    k1 = serving.kappa_for(2, 16, 5)
    assert np.array_equal(k1, serving.kappa_for(2, 16, 5))
    assert k1.shape == (256,) and np.all(k1 > 0)
    assert abs(np.log(k1).std() - 1.0) < 0.15


def _fp(D, n, k, prec, solver=_lib.HDG_SOLVER_PCG):
    b = ctypes.c_double()
    assert _lib.load().hdg_footprint(D, n, k, prec, solver, ctypes.byref(b)) == _lib.HDG_OK
    return b.value


def test_footprint_grows_with_the_problem():
    for prec in (_lib.HDG_PREC_FP64, _lib.HDG_PREC_FF_BLOCK):
        assert _fp(2, 16, 1, prec) < _fp(2, 32, 1, prec) < _fp(2, 32, 2, prec)
        assert _fp(3, 8, 1, prec) < _fp(3, 8, 2, prec) < _fp(3, 16, 2, prec)
    # the FP64 recovery factors [U11 | U12 | y] are larger than the float-float X pair
    assert _fp(3, 16, 2, _lib.HDG_PREC_FP64) > _fp(3, 16, 2, _lib.HDG_PREC_FF_BLOCK)
    # the 32^3 k=2 workload needs on the order of 10-20 GB
    assert 5e9 < _fp(3, 32, 2, _lib.HDG_PREC_FF_BLOCK) < 4e10


def test_footprint_rejects_bad_shapes():
    b = ctypes.c_double()
    lib = _lib.load()
    assert lib.hdg_footprint(4, 8, 1, 0, 0, ctypes.byref(b)) == _lib.HDG_ERR_INVALID
    assert lib.hdg_footprint(2, 0, 1, 0, 0, ctypes.byref(b)) == _lib.HDG_ERR_INVALID
    assert lib.hdg_footprint(2, 8, 5, 0, 0, ctypes.byref(b)) == _lib.HDG_ERR_INVALID


def test_batching_workload_is_seeded():
    from gridaphybrid_gb300.batching import batching_workload
    a, b = batching_workload(seed=4), batching_workload(seed=4)
    assert len(a) == 64
    assert all(x["n"] == y["n"] and x["k"] == y["k"] and np.array_equal(x["kappa"], y["kappa"]) for x, y in zip(a, b))
    assert {x["k"] for x in a} == {1, 2, 3} and all(16 <= x["n"] <= 128 for x in a)
    assert abs(np.log(a[0]["kappa"]).std() - 1.5) < 0.3


def _resp(ticket, status, shape, request, message=b""):
    return {"ticket": ticket, "status": status, "iters": 7, "relres": 1e-3, "latency_ms": 10.0 + ticket,
            "queue_ms": 1.0, "run_ms": 9.0, "reused_mesh": 0, "shape": shape, "request": request,
            "message": message}


def test_latency_summary_lists_failures_with_their_requests():
    resp = [_resp(i, 0, (2, 8, 1), (2, 8, 1, i)) for i in range(9)]
    resp.append(_resp(9, _lib.HDG_ERR_NOT_CONVERGED, (2, 16, 3), (2, 16, 3, 42), b"refined PCG: stalled"))
    s = serving.latency_summary(resp, wall_s=1.0)
    assert s["completed"] == 9 and s["failed"] == 1
    (f,) = s["failures"]
    assert f["request"] == (2, 16, 3, 42)
    assert f["status"] == _lib.HDG_ERR_NOT_CONVERGED and f["iters"] == 7
    assert f["message"] == "refined PCG: stalled"
    # a failed request counts in no latency figure
    assert s["max_ms"] == 18.0


def test_response_struct_matches_the_c_layout():
    """hdg_response: an 8-byte ticket, two ints, seven doubles, two ints, then the 160-byte message."""
    fields = dict(_lib.Response._fields_)
    assert "message" in fields
    assert ctypes.sizeof(_lib.Response) == 8 + 4 + 4 + 8 * 7 + 4 + 4 + 160
