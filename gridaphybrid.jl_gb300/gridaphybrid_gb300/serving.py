"""Serving: HDG solves of different meshes, orders and permeability fields
submitted as they arrive to the library's native request loop
(hdg_server_* in include/hdg_gb300.h).  Workers run admitted requests
concurrently, each on its own stream; meshes stay resident on the GPU and are
reused by later requests of the same shape.  There is no reference
counterpart: the reference solves one problem per ``solve(op)`` call.
"""
import ctypes
import time

import numpy as np

from . import _lib


class Server:
    """A native request loop on one GPU (hdg_server)."""

    def __init__(self, device=0, slots=8, budget_bytes=0.0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        rc = self.lib.hdg_server_create(device, slots, float(budget_bytes), ctypes.byref(h))
        if rc != _lib.HDG_OK:
            raise _lib.HdgError(rc, "hdg_server_create(device=%d) failed" % device)
        self.h = h
        self._keep = {}  # ticket -> (solution buffer, request shape)

    def check(self, rc):
        if rc != _lib.HDG_OK:
            raise _lib.HdgError(rc, self.lib.hdg_server_last_error(self.h).decode())

    @staticmethod
    def sizes(D, n, k):
        """(ncells, ni, nfree) of the Cartesian Darcy problem n^D, order k."""
        k1 = k + 1
        nk = k1 ** D
        nfd = k1 ** (D - 1)
        ncells = n ** D
        nfacets = D * n ** (D - 1) * (n + 1)
        nbnd = 2 * D * n ** (D - 1)
        return ncells, (D + 1) * nk, (nfacets - nbnd) * nfd

    def submit(self, D, n, k, kappa=None, precision=_lib.HDG_PREC_FF_BLOCK, problem=_lib.HDG_PROBLEM_SIN,
               stab=_lib.HDG_STAB_TEXTBOOK, solver=_lib.HDG_SOLVER_PCG, tau=1.0, rtol=1e-10, maxit=20000,
               want_solution=False):
        """Queues one solve; returns its ticket."""
        sol = None
        if want_solution:
            ncells, ni, nfree = self.sizes(D, n, k)
            sol = np.empty(ncells * ni + nfree)
        kap = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
        if kap is not None and kap.size != n ** D:
            raise ValueError("kappa needs n^D values")
        req = _lib.Request(D, n, k, problem, stab, precision, solver, maxit, tau, rtol,
                           None if kap is None else kap.ctypes.data, None if sol is None else sol.ctypes.data)
        t = ctypes.c_longlong()
        self.check(self.lib.hdg_server_submit(self.h, ctypes.byref(req), ctypes.byref(t)))
        self._keep[t.value] = (sol, (D, n, k))
        return t.value

    def poll(self, timeout_ms=0.0, max_items=256):
        """Finished requests as dicts (with 'solution' when it was asked for)."""
        buf = (_lib.Response * max_items)()
        cnt = ctypes.c_int()
        self.check(self.lib.hdg_server_poll(self.h, buf, max_items, float(timeout_ms), ctypes.byref(cnt)))
        out = []
        for i in range(cnt.value):
            r = buf[i]
            d = {f: getattr(r, f) for f, _ in _lib.Response._fields_}
            sol, shape = self._keep.pop(r.ticket, (None, None))
            d["solution"] = sol
            d["shape"] = shape
            out.append(d)
        return out

    def drain(self, timeout_ms=600000.0):
        self.check(self.lib.hdg_server_drain(self.h, float(timeout_ms)))

    def stats(self):
        st = np.zeros(14)
        self.check(self.lib.hdg_server_stats(self.h, _lib.ptr(st)))
        keys = ["submitted", "completed", "failed", "running", "queued", "bytes_in_use", "budget",
                "peak_bytes", "mesh_hits", "mesh_misses", "evictions", "max_concurrent", "busy_ms",
                "retries_after_nomem"]
        return dict(zip(keys, st.tolist()))

    def close(self):
        if getattr(self, "h", None):
            self.lib.hdg_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# The request stream of the serving workload: Poisson arrivals; 2D with
# probability P_2D, n = round(exp(N(ln MU, SIGMA^2))) truncated to the range;
# k uniform; per-cell permeability exp(N(0, 1)).
P_2D = 0.75
N2D_MU, N2D_SIGMA, N2D_RANGE = 32.0, 0.7, (8, 256)
N3D_MU, N3D_SIGMA, N3D_RANGE = 12.0, 0.45, (4, 48)
K2D = (1, 2, 3)
K3D = (1, 2, 3)


def poisson_trace(rate=200.0, seconds=60.0, seed=0):
    """[(arrival_s, D, n, k, kappa_seed)] of the seeded serving workload."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        if rng.random() < P_2D:
            D, (lo, hi), mu, sig, ks = 2, N2D_RANGE, N2D_MU, N2D_SIGMA, K2D
        else:
            D, (lo, hi), mu, sig, ks = 3, N3D_RANGE, N3D_MU, N3D_SIGMA, K3D
        n = int(np.clip(np.rint(np.exp(rng.normal(np.log(mu), sig))), lo, hi))
        k = int(ks[rng.integers(len(ks))])
        out.append((t, D, n, k, int(rng.integers(2 ** 31))))
    return out


def kappa_for(D, n, seed):
    return np.exp(np.random.default_rng(seed).normal(size=n ** D))


def run_trace(server, trace, precision, rtol=1e-10, max_seconds=None, rejected=None):
    """Submits each request at its arrival time; returns (responses, wall
    seconds).  A request the server refuses at submit (its footprint exceeds
    the whole HBM budget) is appended to `rejected` as (D, n, k, message) when
    a list is given, and re-raised otherwise."""
    t0 = time.perf_counter()
    resp = []
    requests = {}  # ticket -> (D, n, k, kappa seed)
    pending = 0
    for (ta, D, n, k, ks) in trace:
        if max_seconds is not None and ta > max_seconds:
            break
        while True:
            now = time.perf_counter() - t0
            if now >= ta:
                break
            resp += server.poll(timeout_ms=0.0)
            time.sleep(min(ta - now, 0.002))
        try:
            ticket = server.submit(D, n, k, kappa=kappa_for(D, n, ks), precision=precision, rtol=rtol)
        except _lib.HdgError as e:
            if rejected is None:
                raise
            rejected.append((D, n, k, str(e)))
            continue
        requests[ticket] = (D, n, k, ks)
        pending += 1
    server.drain()
    resp += server.poll(timeout_ms=0.0, max_items=max(256, pending))
    while len(resp) < pending:
        got = server.poll(timeout_ms=100.0, max_items=256)
        if not got:
            break
        resp += got
    for r in resp:
        r["request"] = requests.get(r["ticket"])
    return resp, time.perf_counter() - t0


def latency_summary(resp, wall_s):
    lat = np.array([r["latency_ms"] for r in resp if r["status"] == 0])
    ok = int(lat.size)
    # each failed request: its shape and kappa seed (to replay it), the status and where the solve stopped
    failures = [{"request": r.get("request"), "status": int(r["status"]), "iters": int(r["iters"]),
                 "relres": float(r["relres"]),
                 "message": r["message"].decode(errors="replace") if isinstance(r.get("message"), bytes) else ""}
                for r in resp if r["status"] != 0][:20]
    if ok == 0:
        return {"completed": 0, "failed": len(resp), "failures": failures}
    cells = sum(r["shape"][1] ** r["shape"][0] for r in resp if r["status"] == 0)
    return {
        "completed": ok, "failed": len(resp) - ok,
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "mean_ms": float(lat.mean()), "max_ms": float(lat.max()),
        "solves_per_s": ok / wall_s, "cells_per_s": cells / wall_s, "wall_s": wall_s,
        "mesh_reuse": float(np.mean([r["reused_mesh"] for r in resp if r["status"] == 0])),
        "queue_p50_ms": float(np.percentile([r["queue_ms"] for r in resp if r["status"] == 0], 50)),
        "run_p50_ms": float(np.percentile([r["run_ms"] for r in resp if r["status"] == 0], 50)),
        "by_class": _by_class(resp),
        "failures": failures,
    }


def _by_class(resp):
    """Per (D, k): completed requests, cells, latency p50/p99 and run time p50."""
    out = {}
    for D, k in sorted({(r["shape"][0], r["shape"][2]) for r in resp if r["status"] == 0}):
        rs = [r for r in resp if r["status"] == 0 and r["shape"][0] == D and r["shape"][2] == k]
        lat = np.array([r["latency_ms"] for r in rs])
        out["%dD_k%d" % (D, k)] = {
            "completed": len(rs), "cells": int(sum(r["shape"][1] ** D for r in rs)),
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "run_p50_ms": float(np.percentile([r["run_ms"] for r in rs], 50)),
        }
    return out
