"""GPU test of hdg_static_condensation_noalloc, the allocation-free variant of
the FP32 + float-float refined condensation for callers that cannot allocate
device memory.

It is called through the C ABI with device buffers (made by the test, not by
the library) and must reproduce hdg_static_condensation(HDG_PREC_FP32_REFINED)
within the refined path's tolerance, on two calls in a row (the second call
finds the shared scratch array holding the first call's contents).  This file
is collected last so that a stop-at-first-failure run has run every other test
first; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from gridaphybrid_gb300 import _lib
from oracle import oracle

pytestmark = pytest.mark.gpu

RTOL_MIXED_CELL = 1e-10


def relmax(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def _reference(ctx, A, b, ni):
    ncells, n, _ = A.shape
    nf = n - ni
    S = np.empty((ncells, nf, nf))
    g = np.empty((ncells, nf))
    info = np.zeros(ncells, dtype=np.int32)
    ctx.check(ctx.lib.hdg_static_condensation(ctx.handle, _lib.HDG_PREC_FP32_REFINED, ncells, ni, nf,
                                              _lib.ptr(A), _lib.ptr(b), _lib.ptr(S), _lib.ptr(g),
                                              _lib.ptr(info)))
    return S, g


def _allocations(ctx):
    n = ctypes.c_longlong()
    ctx.check(ctx.lib.hdg_device_allocations(ctypes.byref(n)))
    return n.value


@pytest.mark.parametrize("D,k,n", [(3, 2, (2, 2, 2)), (2, 3, (4, 3))])
def test_noalloc_matches_allocating_entry_point(D, k, n):
    torch = pytest.importorskip("torch")
    ctx = _lib.Context(0)
    m = oracle.Mesh(D, n, k)
    kappa = np.exp(np.random.default_rng(21).normal(size=m.ncells))
    A, b = m.integrate(problem=oracle.PROBLEM_SIN, kappa=kappa)
    A = np.ascontiguousarray(A)
    b = np.ascontiguousarray(b)
    S_ref, g_ref = _reference(ctx, A, b, m.ni)
    dA = torch.from_numpy(A).cuda()
    db = torch.from_numpy(b).cuda()
    outs = []
    for call in range(2):
        outs.append((torch.full((m.ncells, m.nf, m.nf), float("nan"), dtype=torch.float64, device="cuda"),
                     torch.full((m.ncells, m.nf), float("nan"), dtype=torch.float64, device="cuda"),
                     torch.full((m.ncells,), -7, dtype=torch.int32, device="cuda")))
    torch.cuda.synchronize()
    allocs0 = _allocations(ctx)
    free_after_first = None
    for call, (dS, dg, dinfo) in enumerate(outs):
        dev0 = torch.cuda.current_device()
        rc = ctx.lib.hdg_static_condensation_noalloc(ctx.handle, m.ncells, m.ni, m.nf, _lib.ptr(dA),
                                                     _lib.ptr(db), _lib.ptr(dS), _lib.ptr(dg), _lib.ptr(dinfo))
        assert rc == _lib.HDG_OK, ctx.lib.hdg_last_error(ctx.handle)
        assert torch.cuda.current_device() == dev0
        if call == 0:
            # the first call may load the library's code (and with it the
            # fixed array) onto the device; from then on free memory must not move
            free_after_first = torch.cuda.mem_get_info()[0]
        else:
            assert torch.cuda.mem_get_info()[0] == free_after_first
        S = dS.cpu().numpy()
        g = dg.cpu().numpy()
        assert (dinfo.cpu().numpy() == 0).all()
        assert relmax(S, S_ref) < RTOL_MIXED_CELL, call
        assert relmax(g, g_ref) < RTOL_MIXED_CELL, call
        # and against the FP64 oracle
        S0, g0, _ = oracle.static_condensation(A, b, m.ni)
        assert relmax(S, S0) < RTOL_MIXED_CELL and relmax(g, g0) < RTOL_MIXED_CELL
    # info may be NULL
    dS, dg, _ = outs[0]
    rc = ctx.lib.hdg_static_condensation_noalloc(ctx.handle, m.ncells, m.ni, m.nf, _lib.ptr(dA), _lib.ptr(db),
                                                 _lib.ptr(dS), _lib.ptr(dg), None)
    assert rc == _lib.HDG_OK
    assert relmax(dS.cpu().numpy(), S_ref) < RTOL_MIXED_CELL
    # the library allocated nothing in any of the three calls
    assert _allocations(ctx) == allocs0
    assert torch.cuda.mem_get_info()[0] == free_after_first
    ctx.close()


def _max_cells(n, with_info):
    """Largest batch of n x n cells the fixed array takes: the FP32 hi/lo
    staging of A and b, rounded up to 256 bytes, one 256-byte flag slot, and
    the per-cell info ints when the caller passes info = NULL."""
    scratch = _lib.HDG_NOALLOC_SCRATCH_BYTES
    per_cell = 2 * (n * n + n) * 4

    def need(c):
        return (c * per_cell + 255) // 256 * 256 + 256 + (0 if with_info else 4 * c)

    c = scratch // per_cell
    while need(c) > scratch:
        c -= 1
    assert need(c + 1) > scratch
    return c


@pytest.mark.parametrize("with_info", [True, False])
def test_noalloc_batch_at_the_limit(with_info):
    """A batch exactly at the fixed array's capacity runs and equals the
    allocating path; one cell more is refused before anything runs."""
    torch = pytest.importorskip("torch")
    ctx = _lib.Context(0)
    ni, nf = 12, 8
    n = ni + nf
    ncells = _max_cells(n, with_info)
    rng = np.random.default_rng(5)
    base = rng.normal(size=(16, n, n))
    base[:, np.arange(ni), np.arange(ni)] += 2.0 * np.sqrt(n)
    A = np.ascontiguousarray(base[np.arange(ncells) % 16])
    b = rng.normal(size=(ncells, n))
    S_ref, g_ref = _reference(ctx, A, b, ni)
    dA = torch.from_numpy(A).cuda()
    db = torch.from_numpy(b).cuda()
    dS = torch.full((ncells, nf, nf), float("nan"), dtype=torch.float64, device="cuda")
    dg = torch.full((ncells, nf), float("nan"), dtype=torch.float64, device="cuda")
    dinfo = torch.full((ncells,), -7, dtype=torch.int32, device="cuda") if with_info else None
    torch.cuda.synchronize()
    allocs0 = _allocations(ctx)
    rc = ctx.lib.hdg_static_condensation_noalloc(ctx.handle, ncells, ni, nf, _lib.ptr(dA), _lib.ptr(db),
                                                 _lib.ptr(dS), _lib.ptr(dg), _lib.ptr(dinfo))
    assert rc == _lib.HDG_OK, ctx.lib.hdg_last_error(ctx.handle)
    assert relmax(dS.cpu().numpy(), S_ref) < RTOL_MIXED_CELL
    assert relmax(dg.cpu().numpy(), g_ref) < RTOL_MIXED_CELL
    rc = ctx.lib.hdg_static_condensation_noalloc(ctx.handle, ncells + 1, ni, nf, _lib.ptr(dA), _lib.ptr(db),
                                                 _lib.ptr(dS), _lib.ptr(dg), _lib.ptr(dinfo))
    assert rc == _lib.HDG_ERR_INVALID
    assert b"scratch" in ctx.lib.hdg_last_error(ctx.handle)
    assert _allocations(ctx) == allocs0
    ctx.close()


def test_noalloc_rejects_oversized_batches_and_host_pointers():
    torch = pytest.importorskip("torch")
    ctx = _lib.Context(0)
    ni, nf = 108, 54
    n = ni + nf
    too_many = _max_cells(n, False) + 1
    # the size check comes before any pointer is touched
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = ctx.lib.hdg_static_condensation_noalloc(ctx.handle, too_many, ni, nf, _lib.ptr(dummy), _lib.ptr(dummy),
                                                 _lib.ptr(dummy), _lib.ptr(dummy), None)
    assert rc == _lib.HDG_ERR_INVALID
    assert b"scratch" in ctx.lib.hdg_last_error(ctx.handle)
    A = np.zeros((1, n, n))
    b = np.zeros((1, n))
    S = np.zeros((1, nf, nf))
    g = np.zeros((1, nf))
    rc = ctx.lib.hdg_static_condensation_noalloc(ctx.handle, 1, ni, nf, _lib.ptr(A), _lib.ptr(b), _lib.ptr(S),
                                                 _lib.ptr(g), None)
    assert rc == _lib.HDG_ERR_INVALID
    assert b"device pointers" in ctx.lib.hdg_last_error(ctx.handle)
    ctx.close()
