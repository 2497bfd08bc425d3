"""Benchmark of the hybridization hot path on one GB300.

Workload: 3D Darcy HDG on [0,1]^3, 32x32x32 hexes (32,768 cells), k = 2
(108 interior + 54 facet DOFs per cell), tau = 1, per-cell permeability
lognormal(0, 1) from seed 0, manufactured p = sin(pi x) sin(pi y) sin(pi z),
skeleton PCG to 1e-10 relative residual.  Synthetic inputs (no dataset).

One step = the whole path: integrate + condense every cell, assemble the
skeleton CSR system, facet-block-Jacobi PCG, recover the interiors.

  value : cells / s of a step with inputs resident in HBM (CUDA events on the
          library's stream around K steps).  The step's working set (cell
          blocks, factors, CSR: > 10 GB) is far larger than L2, so no flush is
          needed between steps.
  e2e   : the same metric through hdg_solve() with HOST buffers: permeability
          copied in and the full free-DOF vector copied out every step.

--impl reference times the CPU restatement of the reference (the oracle:
GridapHybrid.jl's Julia path cannot run on this machine: no Julia toolchain)
on all host cores.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "gridaphybrid.jl_gb300"))

N_SIDE = 32
K_ORDER = 2
RTOL = 1e-10
MAXIT = 20000
SEED = 0
METRIC = "HDG cells condensed/s (full integrate+condense+assemble+PCG+recover step)"
UNIT = "cells/s"


def workload_config(precision):
    return {
        "workload": "3D Darcy HDG %dx%dx%d hex, k=2 (108 interior + 54 facet DOFs/cell), tau=1, " % ((N_SIDE,) * 3) +
                    "lognormal(0,1) per-cell permeability seed 0, p=sin(pi x)sin(pi y)sin(pi z), "
                    "skeleton PCG to 1e-10",
        "cells": N_SIDE ** 3,
        "precision": precision,
        "l2": "working set > L2 (cell blocks + factors + CSR ~ 13 GB); no flush needed",
    }


def kappa_field():
    return np.exp(np.random.default_rng(SEED).normal(0.0, 1.0, N_SIDE ** 3))


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def oracle_setup():
    """The oracle's once-per-mesh work (topology, facet DOFs, Dirichlet values,
    CSR pattern) for the workload, timed on its own."""
    from oracle import oracle

    t0 = time.perf_counter()
    setup = oracle.DarcySetup(3, K_ORDER, (N_SIDE,) * 3, problem=oracle.PROBLEM_SIN)
    return setup, time.perf_counter() - t0


def cpu_baseline_sample(setup, setup_s):
    """The oracle (C, FP64, OpenMP) on the host cores: one 32^3 solve on a
    mesh set up beforehand, the same per-solve work the GPU step times."""
    from oracle import oracle

    nthreads = oracle.max_threads()
    kappa = kappa_field()
    t0 = time.perf_counter()
    r = setup.step(tau=1.0, stab=oracle.STAB_TEXTBOOK, kappa=kappa, solver=1, rtol=RTOL, maxit=MAXIT,
                   want_solution=False)
    dt = time.perf_counter() - t0
    return {
        "value": N_SIDE ** 3 / dt,
        "unit": UNIT,
        "cores": nthreads,
        "kind": "port",
        "sample": "one full %d^3 k=2 solve (integrate+condense, assemble, block-Jacobi PCG %d its to %g, "
                  "re-integrate + backward map as the reference does) in %.2f s, on a mesh set up beforehand "
                  "(set-up %.2f s, not timed, like the GPU problem creation)" % (N_SIDE, r["iters"], RTOL, dt,
                                                                                  setup_s),
        "solver": "block-Jacobi PCG on the assembled FP64 CSR (the reference solves with sparse direct A\\b, "
                  "src/HybridAffineFEOperators.jl:74)",
        "setup_s": setup_s,
        "phases_s": {k: round(float(v), 3) for k, v in zip(
            ["integrate_condense", "assemble", "solve", "recover", "total"], r["times"])},
    }


def run_reference(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from oracle import oracle

    oracle.build()
    kappa = kappa_field()
    setup, setup_s = oracle_setup()
    times = []
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        r = setup.step(tau=1.0, stab=oracle.STAB_TEXTBOOK, kappa=kappa, solver=1, rtol=RTOL, maxit=MAXIT,
                       want_solution=False)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
    setup.close()
    ms = 1000.0 * statistics.mean(times)
    value = N_SIDE ** 3 / (ms / 1000.0)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config("fp64"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.max_threads(), "kind": "port",
                         "sample": "full %d^3 k=2 solve per step on a mesh set up once before the timed steps "
                                   "(set-up %.2f s: topology, facet DOFs, Dirichlet values, CSR pattern); C "
                                   "restatement of the reference path (Julia/Gridap are not installed on this "
                                   "machine)" % (N_SIDE, setup_s),
                         "solver": "block-Jacobi PCG on the assembled FP64 CSR (the reference solves with sparse "
                                   "direct A\\b, src/HybridAffineFEOperators.jl:74)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "setup_s": setup_s,
        "pcg_iters": r["iters"],
    }
    print(json.dumps(line))


def run_serving(args, prec, prec64):
    """The serving workload: a seeded Poisson stream of 2D/3D Darcy solves of
    different sizes, orders and permeability fields submitted at their arrival
    times to the native request loop; p50/p99 latency and solves/s, for the
    selected precision and (over the first part of the same stream) the plain
    FP64 path."""
    from gridaphybrid_gb300 import serving
    trace = serving.poisson_trace(rate=args.serve_rate, seconds=args.serve_seconds, seed=0)
    out = {
        "workload": "Poisson %.0f req/s for %.0f s (seed 0): 2D with p=%.2f, n=round(exp(N(ln %g, %g^2))) in "
                    "[%d,%d], k in %s; 3D n=round(exp(N(ln %g, %g^2))) in [%d,%d], k in %s; kappa=exp(N(0,1)) "
                    "per cell; PCG to 1e-10" % (
                        args.serve_rate, args.serve_seconds, serving.P_2D, serving.N2D_MU, serving.N2D_SIGMA,
                        *serving.N2D_RANGE, list(serving.K2D), serving.N3D_MU, serving.N3D_SIGMA,
                        *serving.N3D_RANGE, list(serving.K3D)),
        "requests": len(trace), "slots": args.serve_slots,
    }
    runs = [(args.precision, prec, None)]
    if args.precision != "fp64" and args.serve_fp64_seconds > 0:
        runs.append(("fp64", prec64, args.serve_fp64_seconds))
    for name, p, limit in runs:
        rejected = []
        with serving.Server(slots=args.serve_slots) as srv:
            resp, wall = serving.run_trace(srv, trace, p, max_seconds=limit, rejected=rejected)
            st = srv.stats()
        summ = serving.latency_summary(resp, wall)
        summ["rejected_over_budget"] = [list(r[:3]) for r in rejected]
        summ.update({"seconds_of_trace": limit or args.serve_seconds, "peak_hbm_gb": st["peak_bytes"] / 1e9,
                     "max_concurrent": int(st["max_concurrent"]), "mesh_hits": int(st["mesh_hits"]),
                     "evictions": int(st["evictions"]), "retries_after_nomem": int(st["retries_after_nomem"])})
        out[name] = summ
    return out


def run_batching(args, ctx):
    """The batching workload: 64 independent 2D Darcy HDG problems, n ~ U{16..128}
    per side, k ~ U{1,2,3}, kappa = exp(N(0, 1.5^2)) per cell (seed 0).  Each
    (D, k) class is integrated and condensed by one persistent fused launch
    (tile autotuned, launch sequence replayed as a CUDA graph); compared with
    assembling the problems one by one, in FP64 and in float-float."""
    import gridaphybrid_gb300 as gh
    from gridaphybrid_gb300 import _lib
    from gridaphybrid_gb300.batching import Batch, batching_workload
    specs = batching_workload(nproblems=args.batch_problems, seed=0)
    out = {"workload": "%d 2D Darcy HDG problems, n~U{16..128}, k~U{1,2,3}, kappa=exp(N(0,1.5^2)) per cell, "
                       "seed 0" % len(specs)}
    reps = 3
    with Batch(specs, context=ctx) as b:
        out["cells"] = b.cells
        for name, prec in (("ffblock", _lib.HDG_PREC_FF_BLOCK), ("fp64", _lib.HDG_PREC_FP64)):
            b.assemble(prec)   # tune + capture
            b.assemble(prec)
            ctx.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                b.assemble(prec)
            ctx.synchronize()
            batched_ms = 1000.0 * (time.perf_counter() - t0) / reps
            tm = b.timings()
            t0 = time.perf_counter()
            its, rel = b.solve(rtol=RTOL)
            solve_ms = 1000.0 * (time.perf_counter() - t0)
            # the same problems assembled one call each (separate integrate / condense kernels)
            for pb in b.pbs:
                ctx.check(ctx.lib.hdg_assemble(pb.h, prec, None))
            ctx.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                for pb in b.pbs:
                    ctx.check(ctx.lib.hdg_assemble(pb.h, prec, None))
            ctx.synchronize()
            single_ms = 1000.0 * (time.perf_counter() - t0) / reps
            out[name] = {
                "batched_assemble_ms": batched_ms,
                "fused_integrate_condense_ms": tm["fused_integrate_condense_ms"],
                "skeleton_assembly_ms": tm["skeleton_assembly_ms"],
                "cells_condensed_per_s": b.cells / (tm["fused_integrate_condense_ms"] / 1000.0),
                "one_by_one_assemble_ms": single_ms,
                "batched_speedup": single_ms / batched_ms,
                "solve_recover_ms": solve_ms, "pcg_iters_total": int(its.sum()),
                "tuning": b.tuning(prec),
            }
    out["ffblock_vs_fp64_fused"] = (out["fp64"]["fused_integrate_condense_ms"] /
                                    out["ffblock"]["fused_integrate_condense_ms"])
    return out


def run_elasticity(args, ctx):
    """The precision workload: 3D linear elasticity HDG on the unit cube,
    E = 1, nu ~ U(0.2, 0.45) per cell (seed 0), u = (sin pi x, cos pi y, xyz),
    tau = 1/h, cell order k (default 2: n = 405 DOFs per cell).  The fast path
    (float-float block elimination on the FP32 pipes + FP32 skeleton PCG with
    FP64 residual refinement; at k = 1 also the FP32 LU + refinement path)
    against the plain FP64 path on the GPU (FP64 block elimination at k = 2,
    where the cell block exceeds the shared-memory LU), all solved to 1e-12."""
    import gridaphybrid_gb300 as gh
    from gridaphybrid_gb300 import _lib
    n, k = args.elasticity_n, args.elasticity_k
    nk, nfs = (k + 1) ** 3, (k + 1) ** 2
    nu = np.random.default_rng(0).uniform(0.2, 0.45, size=n ** 3)
    model = gh.CartesianDiscreteModel((0, 1) * 3, (n,) * 3)
    X, Y = gh.elasticity_spaces(model, k)
    out = {"workload": "3D linear elasticity HDG %d^3 hex, k=%d (sym stress 6x%d + displacement 3x%d inside, "
                       "3x%d per facet, n=%d per cell), E=1, nu~U(0.2,0.45) per cell, u=(sin pi x, cos pi y, xyz), "
                       "tau=1/h" % (n, k, nk, nk, nfs, 9 * nk + 18 * nfs),
           "cells": n ** 3}
    paths = [("fp64", _lib.HDG_PREC_FP64), ("ffblock", _lib.HDG_PREC_FF_BLOCK)]
    if k == 1:
        paths.append(("fp32_refined", _lib.HDG_PREC_FP32_REFINED))
    sols = {}
    for name, prec in paths:
        form = gh.ElasticityHDG(nu=nu, problem="smooth")
        op = gh.HybridAffineFEOperator(form, X, Y, [1, 2], [3], precision=prec, context=ctx)
        xh = gh.solve(op, solver="pcg", rtol=1e-12)
        h = op.pb.h
        reps = 2
        phases = np.zeros(5)
        t0 = time.perf_counter()
        for _ in range(reps):
            ctx.check(ctx.lib.hdg_assemble(h, prec, None))
            it, rel = ctypes.c_int(), ctypes.c_double()
            ctx.check(ctx.lib.hdg_solve_skeleton(h, _lib.HDG_SOLVER_PCG, 1e-10, 20000, ctypes.byref(it),
                                                 ctypes.byref(rel)))
            ctx.check(ctx.lib.hdg_recover(h))
            ms5 = np.zeros(5)
            ctx.check(ctx.lib.hdg_get_timings(h, _lib.ptr(ms5)))
            phases += ms5
        ctx.synchronize()
        ms = 1000.0 * (time.perf_counter() - t0) / reps
        phases /= reps
        es, eu = xh.l2_errors()
        sols[name] = xh.free_dof_values.copy()
        out[name] = {"ms_per_solve": ms, "cells_per_s": n ** 3 / (ms / 1000.0), "pcg_iters": xh.iterations,
                     "phase_ms": {"integrate": phases[0], "condense": phases[1], "assemble": phases[2],
                                  "solve": phases[3], "recover": phases[4]},
                     "err_sigma_vs_exact": es, "err_u_vs_exact": eu}
        op.pb.close()
    ref = sols["fp64"]
    for name, _ in paths[1:]:
        out[name]["rel_err_vs_fp64"] = float(np.abs(sols[name] - ref).max() / np.abs(ref).max())
        out[name]["speedup_vs_fp64"] = out["fp64"]["ms_per_solve"] / out[name]["ms_per_solve"]
    return out


def run_skewed(args, ctx):
    """The headline workload on an affine mesh whose cells are not
    axis-aligned: the 32^3 Cartesian topology with every cell mapped by one
    global skew x -> B x (hdg_problem_create, Gridap-style arrays), so the
    integration and the block elimination take their general-Jacobian paths
    (every flux component couples to every facet).  Same form, kappa and
    solver tolerance; the float-float path timed, and compared once with the
    plain FP64 path on the same mesh."""
    from gridaphybrid_gb300 import _lib
    lib = ctx.lib
    n, D, k = args.skewed_n, 3, K_ORDER
    B = np.array([[1.0, 0.3, 0.1], [0.1, 1.0, 0.2], [0.05, 0.1, 1.0]])
    base = ctypes.c_void_p()
    cells = np.array([n] * 3, dtype=np.int32)
    dom = np.array([0, 1, 0, 1, 0, 1], dtype=np.float64)
    ctx.check(lib.hdg_problem_create_cartesian(ctx.handle, D, _lib.ptr(cells), _lib.ptr(dom), k, ctypes.byref(base)))
    info = np.zeros(8, dtype=np.int64)
    ctx.check(lib.hdg_problem_info(base, _lib.ptr(info)))
    ncells, nfacets, nfd = int(info[0]), int(info[1]), int(info[7])
    cf = np.empty((ncells, 2 * D), dtype=np.int32)
    fd = np.empty((nfacets, nfd), dtype=np.int32)
    ctx.check(lib.hdg_get_topology(base, _lib.ptr(cf), None, _lib.ptr(fd)))
    lib.hdg_problem_destroy(base)
    idx = np.stack(np.unravel_index(np.arange(ncells), (n, n, n), order="F"), axis=1).astype(np.float64)
    origin = np.ascontiguousarray((idx / n) @ B.T)
    jac = np.ascontiguousarray(np.broadcast_to((B / n).T, (ncells, D, D)))  # per cell, column-major
    h = ctypes.c_void_p()
    ctx.check(lib.hdg_problem_create(ctx.handle, D, k, ncells, nfacets, _lib.ptr(origin), _lib.ptr(jac), _lib.ptr(cf),
                                     _lib.ptr(fd), ctypes.byref(h)))
    ctx.check(lib.hdg_set_darcy(h, _lib.HDG_STAB_TEXTBOOK, 1.0, _lib.HDG_PROBLEM_SIN))
    kappa = np.exp(np.random.default_rng(SEED).normal(0.0, 1.0, ncells))  # the headline's field at n = 32
    ctx.check(lib.hdg_set_permeability(h, _lib.ptr(kappa)))
    ctx.check(lib.hdg_problem_info(h, _lib.ptr(info)))
    ni, nfree = int(info[2]), int(info[4])

    def run(prec, rtol):
        ctx.check(lib.hdg_assemble(h, prec, None))
        it, rel = ctypes.c_int(), ctypes.c_double()
        ctx.check(lib.hdg_solve_skeleton(h, _lib.HDG_SOLVER_PCG, rtol, MAXIT, ctypes.byref(it), ctypes.byref(rel)))
        ctx.check(lib.hdg_recover(h))
        return it.value

    out = {"workload": "the %d^3 k=2 Darcy workload with every cell mapped by the skew B = %s (non-diagonal "
                       "Jacobians: general-Jacobian integration and elimination)" % (n, B.tolist()),
           "cells": ncells}
    sols = {}
    for name, prec in (("fp64", _lib.HDG_PREC_FP64), ("ffblock", _lib.HDG_PREC_FF_BLOCK)):
        run(prec, 1e-12)
        sol = np.empty(ncells * ni + nfree)
        ctx.check(lib.hdg_get_free_dof_values(h, _lib.ptr(sol)))
        sols[name] = sol
        if name == "ffblock":
            for _ in range(args.warmup):
                run(prec, RTOL)
            ctx.synchronize()
            ctx.check(lib.hdg_context_record(ctx.handle, 0))
            phase, its = np.zeros(5), []
            for _ in range(args.steps):
                its.append(run(prec, RTOL))
                t = np.zeros(5)
                lib.hdg_get_timings(h, _lib.ptr(t))
                phase += t
            ctx.check(lib.hdg_context_record(ctx.handle, 1))
            ctx.synchronize()
            ms = ctypes.c_double()
            ctx.check(lib.hdg_context_elapsed_ms(ctx.handle, 0, 1, ctypes.byref(ms)))
            step_ms = ms.value / args.steps
            out[name] = {"ms_per_step": step_ms, "cells_per_s": ncells / (step_ms / 1000.0),
                         "phases_ms": dict(zip(["integrate", "condense", "assemble", "skeleton_pcg", "recover"],
                                               [float(x) for x in phase / args.steps])),
                         "pcg_iters": statistics.mean(its)}
    ref = sols["fp64"]
    out["ffblock"]["rel_err_vs_fp64"] = float(np.abs(sols["ffblock"] - ref).max() / np.abs(ref).max())
    lib.hdg_problem_destroy(h)
    return out


ERR_GATE = 1e-8


def oracle_accuracy(setup, got, ncells, ni):
    """The selected path's free DOF values (solved to 1e-12) against the
    oracle's (the reference path restated in C, FP64, PCG to 1e-13): max
    relative difference over all free DOFs, in Gridap's layout [flux | pressure
    | skeleton]."""
    from oracle import oracle

    t0 = time.perf_counter()
    r = setup.step(tau=1.0, stab=oracle.STAB_TEXTBOOK, kappa=kappa_field(), solver=1, rtol=1e-13, maxit=MAXIT)
    dt = time.perf_counter() - t0
    nq = 3 * (K_ORDER + 1) ** 3  # flux DOFs per cell
    ref = np.concatenate([r["uint"][:, :nq].ravel(), r["uint"][:, nq:].ravel(), r["lam"]])
    err = float(np.abs(got - ref).max() / np.abs(ref).max())
    return {"rel_err_vs_oracle": err,
            "note": "max |x - x_oracle| / max |x_oracle| over all %d free DOFs; this path solved to 1e-12, the "
                    "oracle (C FP64 restatement of the reference path) by block-Jacobi PCG to 1e-13 in %.1f s"
                    % (len(ref), dt),
            "oracle_pcg_iters": r["iters"], "l2_err_flux_oracle": r["err_flux"], "l2_err_pres_oracle": r["err_pres"]}


# FP32-pipe work of the float-float condensation per cell: thread-level FP32
# operations (FFMA counted twice, FADD and FMUL once) that ncu counts for one
# launch of condense_ffblock_kernel<3,27,9> at 24^3, divided by its cells (the
# kernel does the same work in every cell).  Refreshed with the capture in
# profiles/condense_ffblock_kernel_24cube_k2.md.
# FP32 work of condense_ffblock_kernel<3,27,9> per cell, from an ncu capture at
# 24^3: FADD + FMUL + 2 FFMA thread-instructions per cell (FFMA counts 2 flops)
FFBLOCK_FP32_FLOP_PER_CELL = 3.17e6


def condense_roofline(phase, ncells, peaks):
    """Compute roofline of the condensation: the algorithmic FP64 flops of
    the reference's StaticCondensationMap per cell (2/3 ni^3 + 2 ni^2 nf +
    2 nf^2 ni + 2 ni^2 + 2 ni nf) over the event-timed condensation, against
    the measured FP64 peak (how far past native FP64 the float-float path
    goes), and, where the FP32 work per cell is known from ncu, the FP32-pipe
    fraction."""
    ni, nf = 108, 54
    alg = 2.0 / 3.0 * ni ** 3 + 2 * ni * ni * nf + 2 * nf * nf * ni + 2 * ni * ni + 2 * ni * nf
    ms = float(phase[1])
    ach = alg * ncells / (ms * 1e-3) / 1e12
    out = {"bound": "fp32 pipe (float-float); issue- and latency-limited (ncu: 58 % issue active)",
           "kernel": "condense_ffblock_kernel<3,27,9>", "ms_per_launch": ms,
           "alg_fp64_flop_per_cell": alg, "achieved_fp64_equiv_tflops": ach,
           "fp64_peak_tflops": peaks["fp64_tflops"], "frac_of_fp64_peak": ach / peaks["fp64_tflops"]}
    if FFBLOCK_FP32_FLOP_PER_CELL:
        a32 = FFBLOCK_FP32_FLOP_PER_CELL * ncells / (ms * 1e-3) / 1e12
        out.update({"fp32_flop_per_cell_ncu": FFBLOCK_FP32_FLOP_PER_CELL, "achieved_fp32_tflops": a32,
                    "fp32_peak_tflops": peaks["fp32_tflops"], "frac": a32 / peaks["fp32_tflops"]})
    return out


def run_gpu(args, rank=0, nranks=1, device=0):
    """One replica per GPU: every rank runs the whole workload on its own GPU;
    the timed regions are bracketed by barriers and the maximum over ranks is
    reported.  Rank 0 alone adds the FP64 comparison, serving and CPU baseline."""
    import gridaphybrid_gb300 as gh
    from gridaphybrid_gb300 import _lib, replicas

    precs = {"fp64": _lib.HDG_PREC_FP64, "mixed": _lib.HDG_PREC_FP32_REFINED, "ffblock": _lib.HDG_PREC_FF_BLOCK}
    prec = precs[args.precision]
    ctx = gh.Context(device)
    lib = ctx.lib
    h = ctypes.c_void_p()
    cells = np.array([N_SIDE] * 3, dtype=np.int32)
    dom = np.array([0, 1, 0, 1, 0, 1], dtype=np.float64)
    kappa = kappa_field()
    # problem creation (host mesh, facet numbering, CSR pattern and block maps,
    # uploads), once per mesh like the reference's Skeleton + FE spaces; timed
    # on its own, outside the steps
    ctx.synchronize()
    t_setup = time.perf_counter()
    ctx.check(lib.hdg_problem_create_cartesian(ctx.handle, 3, _lib.ptr(cells), _lib.ptr(dom), K_ORDER,
                                               ctypes.byref(h)))
    ctx.check(lib.hdg_set_darcy(h, _lib.HDG_STAB_TEXTBOOK, 1.0, _lib.HDG_PROBLEM_SIN))
    ctx.check(lib.hdg_set_permeability(h, _lib.ptr(kappa)))
    ctx.synchronize()
    setup_ms = 1000.0 * (time.perf_counter() - t_setup)
    info = np.zeros(8, dtype=np.int64)
    ctx.check(lib.hdg_problem_info(h, _lib.ptr(info)))
    ncells, nfacets, ni, nf, nfree, ndir, nnz, nfd = (int(v) for v in info)

    def step(p, rtol=RTOL):
        ctx.check(lib.hdg_assemble(h, p, None))
        it = ctypes.c_int()
        rel = ctypes.c_double()
        ctx.check(lib.hdg_solve_skeleton(h, _lib.HDG_SOLVER_PCG, rtol, MAXIT, ctypes.byref(it), ctypes.byref(rel)))
        ctx.check(lib.hdg_recover(h))
        return it.value, rel.value

    def timed(p, steps):
        ctx.synchronize()
        replicas.barrier()
        l0 = ctx.launches
        ctx.check(lib.hdg_context_record(ctx.handle, 0))
        phase = np.zeros(5)
        its = []
        rel = None
        for _ in range(steps):
            it, rel = step(p)
            its.append(it)
            t = np.zeros(5)
            lib.hdg_get_timings(h, _lib.ptr(t))
            phase += t
        ctx.check(lib.hdg_context_record(ctx.handle, 1))
        ctx.synchronize()
        replicas.barrier()
        ms = ctypes.c_double()
        ctx.check(lib.hdg_context_elapsed_ms(ctx.handle, 0, 1, ctypes.byref(ms)))
        return (replicas.max_over_ranks(ms.value) / steps, phase / steps, statistics.mean(its), rel,
                ctx.launches - l0)

    for _ in range(args.warmup):
        step(prec)
    sampler = ClockSampler()
    sampler.start()
    ms, phase, mean_iters, rel, launches = timed(prec, args.steps)
    clocks = sampler.stop()

    # kernel timings on this precision's buffers (dominant HBM kernel: the SpMV)
    spmv_ms, asm_ms, cond_ms = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    ctx.check(lib.hdg_time_kernel(h, 3, 20, ctypes.byref(spmv_ms)))
    ctx.check(lib.hdg_time_kernel(h, 2, 5, ctypes.byref(asm_ms)))
    ctx.check(lib.hdg_time_kernel(h, 1, 2, ctypes.byref(cond_ms)))

    # measured FMA pipe peaks (the denominators of the condensation's compute roofline)
    p32, p64 = ctypes.c_double(), ctypes.c_double()
    ctx.check(lib.hdg_measure_pipe_peaks(ctx.handle, ctypes.byref(p32), ctypes.byref(p64)))
    pipe_peaks = {"fp32_tflops": p32.value, "fp64_tflops": p64.value,
                  "how": "FMA chains at full occupancy, CUDA events, this run (an FMA counts 2 flops)"}

    # the selected path solved to 1e-12: its error against the oracle and the
    # plain FP64 GPU path is reported and gated
    got = None
    if rank == 0:
        step(prec, rtol=1e-12)
        got = np.empty(ncells * ni + nfree)
        ctx.check(lib.hdg_get_free_dof_values(h, _lib.ptr(got)))

    # the plain FP64 GPU path on the same workload, and the accuracy of the
    # selected path against it (both solved to 1e-12)
    compare = None
    if args.precision != "fp64" and not args.no_fp64_compare and rank == 0:
        step(precs["fp64"])
        ms64, phase64, iters64, _, _ = timed(precs["fp64"], max(1, min(args.steps, 2)))
        step(precs["fp64"], rtol=1e-12)
        ref = np.empty(ncells * ni + nfree)
        ctx.check(lib.hdg_get_free_dof_values(h, _lib.ptr(ref)))
        compare = {
            "fp64_ms_per_step": ms64,
            "fp64_phases_ms": dict(zip(["integrate", "condense", "assemble", "skeleton_pcg", "recover"],
                                       [float(x) for x in phase64])),
            "speedup_vs_fp64_gpu": ms64 / ms,
            "rel_err_vs_fp64": float(np.abs(got - ref).max() / np.abs(ref).max()),
            "rel_err_note": "max |x - x_fp64| / max |x_fp64| over all free DOFs, both solved to 1e-12",
        }

    # end to end through hdg_solve with host (pinned) buffers
    e2e = None
    if args.e2e_steps > 0:
        try:
            import torch
            kap_h = torch.from_numpy(kappa.copy()).pin_memory()
            out_h = torch.empty(ncells * ni + nfree, dtype=torch.float64).pin_memory()
            pinned = True
        except Exception:
            kap_h = kappa.copy()
            out_h = np.empty(ncells * ni + nfree)
            pinned = False
        kp, op = _lib.ptr(kap_h), _lib.ptr(out_h)
        stats = np.zeros(7)
        ctx.check(lib.hdg_solve(h, prec, _lib.HDG_SOLVER_PCG, RTOL, MAXIT, kp, op, _lib.ptr(stats)))
        replicas.barrier()
        t0 = time.perf_counter()
        for i in range(args.e2e_steps):
            ctx.check(lib.hdg_solve(h, prec, _lib.HDG_SOLVER_PCG, RTOL, MAXIT, kp, op, _lib.ptr(stats)))
        ctx.synchronize()
        replicas.barrier()
        e2e_s = replicas.max_over_ranks(time.perf_counter() - t0) / args.e2e_steps
        e2e = {"value": nranks * ncells / e2e_s, "unit": UNIT, "h2d_bytes_per_step": ncells * 8,
               "d2h_bytes_per_step": (ncells * ni + nfree) * 8, "ms_per_step": e2e_s * 1000.0,
               "host_buffers": "pinned" if pinned else "pageable"}

    if rank != 0:
        lib.hdg_problem_destroy(h)
        return
    batching_out = run_batching(args, ctx) if args.batch_problems > 0 else None
    elasticity_out = run_elasticity(args, ctx) if args.elasticity_n > 0 else None
    skewed_out = run_skewed(args, ctx) if args.skewed_n > 0 else None
    serving_out = run_serving(args, prec, precs["fp64"]) if args.serve_seconds > 0 else None

    peaks, peak_kind = measured_peaks()
    hbm = float(peaks["hbm_gbs"])
    # SpMV of the PCG iterations.  FP64 path: CSR values + one column list per
    # facet block row + two row pointers per block row + z and p_old gathered
    # once + p_new and q written once.  Fast paths (unassembled FP32 cell
    # operator): the cell records (facet blocks above the diagonal, padded to 16 bytes) +
    # the cell->block-row map + z and p_old read once + p_new written once +
    # the per-cell products written.
    nblockrows = nfree // nfd
    nl = 6
    if args.precision == "fp64":
        spmv_bytes = nnz * 8 + (nnz // nfd) * 4 + nblockrows * 16 + 4 * nfree * 8
        spmv_kernel = "pcg_spmv_kernel<double,9>"
        spmv_traffic = None  # not captured
    else:
        bstride = {9: 85, 27: 731}.get(nfd, nfd * nfd)  # blocks padded against bank conflicts
        rec = (nl * (nl - 1) // 2 * bstride + 3) // 4 * 4  # the blocks above the diagonal
        spmv_bytes = ncells * rec * 4 + ncells * nl * 4 + 3 * nfree * 4 + ncells * nf * 4
        spmv_kernel = "cell_spmv32_kernel<6,9>"
        # DRAM read + write of one launch from an ncu capture at 24^3 (73.78 + 1.15 MB
        # over 13,824 cells, the bench configuration), scaled by cells: the kernel
        # streams each cell record once, so traffic grows with the cells
        spmv_traffic = 74.93e6 / 13824 * ncells
    spmv_gbs = spmv_bytes / (spmv_ms.value * 1e-3) / 1e9
    # assembly: condensed blocks + vectors read, CSR values + rhs written
    asm_bytes = ncells * (nf * nf + nf) * 8 + nnz * 8 + nfree * 8
    asm_gbs = asm_bytes / (asm_ms.value * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": nranks * ncells / (ms / 1000.0), "unit": UNIT, "n_gpus": nranks,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "mixed": "f32+ff-refined", "ffblock": "ff(2xf32)+f32-pcg"}[args.precision],
        "data": "synthetic", "config": workload_config(args.precision),
        "phases_ms": dict(zip(["integrate", "condense", "assemble", "skeleton_pcg", "recover"],
                              [float(x) for x in phase])),
        "condense_cells_per_s": ncells / ((phase[0] + phase[1]) / 1000.0),
        "pcg_iters": mean_iters, "pcg_relres": rel, "full_solve_ms": ms,
        "roofline": {"bound": "hbm",
                     "kernel": spmv_kernel,
                     "achieved": spmv_gbs, "peak": hbm,
                     "unit": "GB/s", "frac": spmv_gbs / hbm, "traffic": spmv_traffic, "peak_source": peak_kind,
                     "bytes_per_launch": spmv_bytes, "ms_per_launch": spmv_ms.value},
        "assembly_roofline": {"bound": "hbm", "achieved": asm_gbs, "peak": hbm, "unit": "GB/s",
                              "frac": asm_gbs / hbm, "bytes_per_launch": asm_bytes, "ms_per_launch": asm_ms.value},
        "condense_ms_per_launch": cond_ms.value,
        "clocks": clocks, "e2e": e2e, "gpu_launches": launches,
    }
    if compare:
        line["fp64_compare"] = compare
    if batching_out:
        line["batching"] = batching_out
    if elasticity_out:
        line["elasticity"] = elasticity_out
    if skewed_out is not None:
        line["skewed_mesh"] = skewed_out
    if serving_out:
        line["serving"] = serving_out
    line["setup_ms"] = setup_ms
    line["setup_note"] = ("GPU problem creation (host mesh, numbering, CSR pattern, block maps, uploads), once "
                          "per mesh, outside the timed steps; the CPU arms likewise set up outside their timing")
    line["peaks"] = pipe_peaks
    line["condense_roofline"] = condense_roofline(phase, ncells, pipe_peaks)
    gate_failed = False
    if not args.no_oracle_check or not args.no_cpu_baseline:
        setup, setup_s = oracle_setup()
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline_sample(setup, setup_s)
        if not args.no_oracle_check:
            acc = oracle_accuracy(setup, got, ncells, ni)
            if compare:
                acc["rel_err_vs_fp64_gpu"] = compare["rel_err_vs_fp64"]
            gate_failed = max(acc["rel_err_vs_oracle"], acc.get("rel_err_vs_fp64_gpu", 0.0)) > ERR_GATE
            acc["gate"] = ERR_GATE
            acc["gate_passed"] = not gate_failed
            line["accuracy"] = acc
        setup.close()
    print(json.dumps(line))
    lib.hdg_problem_destroy(h)
    if gate_failed:
        print("error gate failed: the solution differs from the FP64 oracle or the FP64 GPU path by more than "
              "%g (relative)" % ERR_GATE, file=sys.stderr)
        sys.exit(3)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="ffblock", choices=["fp64", "mixed", "ffblock"],
                    help="fp64: plain FP64 path; mixed: FP32 LU + float-float refinement; "
                         "ffblock: Darcy block elimination in float-float (both fast paths use the FP32 "
                         "inner PCG with FP64 residual refinement)")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-oracle-check", action="store_true",
                    help="skip the solution's comparison with the FP64 oracle (and its 1e-8 gate)")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="length of the serving stream (0 skips serving)")
    ap.add_argument("--serve-fp64-seconds", type=float, default=20.0,
                    help="part of the stream replayed on the plain FP64 path")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-slots", type=int, default=16)
    ap.add_argument("--batch-problems", type=int, default=64,
                    help="problems of the batching workload (0 skips it)")
    ap.add_argument("--skewed-n", type=int, default=32,
                    help="cells per side of the skewed-mesh run of the headline form (0: skip)")
    ap.add_argument("--elasticity-n", type=int, default=24,
                    help="cells per side of the elasticity precision workload (0 skips it)")
    ap.add_argument("--elasticity-k", type=int, default=2, choices=(1, 2),
                    help="cell order of the elasticity precision workload")
    ap.add_argument("--n-side", type=int, default=32,
                    help="cells per side (32 is the benchmark workload; smaller sizes are for profiling)")
    args = ap.parse_args()
    global N_SIDE
    N_SIDE = args.n_side
    if args.impl == "reference":
        run_reference(args)
        return
    from gridaphybrid_gb300 import replicas
    # replicas only: each rank solves the whole workload on its own GPU
    rank, nranks, local = replicas.init()
    run_gpu(args, rank=rank, nranks=nranks, device=local)
    replicas.finalize()


if __name__ == "__main__":
    main()
