"""CPU checks of the host-side Map mirror (no device calls)."""
import numpy as np
import pytest

import gridaphybrid_gb300 as gh


def test_scalar2arrayblock_map_reference_test():
    """test/Scalar2ArrayBlockMapTests.jl: bs = [8, 16], blocks are A's and b's sub-ranges."""
    bs = [8, 16]
    rng = np.random.default_rng(0)
    A = rng.random((sum(bs), sum(bs)))
    b = rng.random(sum(bs))
    k = gh.Scalar2ArrayBlockMap()
    cache = gh.return_cache(k, (A, b), bs)
    Ab, bb = gh.evaluate(cache, k, (A, b), bs)
    assert np.array_equal(Ab.array[0, 0], A[0:8, 0:8])
    assert np.array_equal(Ab.array[1, 0], A[8:24, 0:8])
    assert np.array_equal(Ab.array[0, 1], A[0:8, 8:24])
    assert np.array_equal(Ab.array[1, 1], A[8:24, 8:24])
    assert np.array_equal(bb.array[0], b[0:8]) and np.array_equal(bb.array[1], b[8:24])
    assert Ab.touched.all() and bb.touched.all()


def test_scalar2arrayblock_map_three_fields_and_cache_reuse():
    """Three fields, the A, b, bs call form, and a cache reused for a second cell."""
    bs = [3, 5, 2]
    n = sum(bs)
    k = gh.Scalar2ArrayBlockMap()
    rng = np.random.default_rng(1)
    A1, b1 = rng.random((n, n)), rng.random(n)
    A2, b2 = rng.random((n, n)), rng.random(n)
    cache = gh.return_cache(k, A1, b1, bs)
    Ab, bb = gh.evaluate(cache, k, A1, b1, bs)
    assert np.array_equal(np.block([[Ab.array[i, j] for j in range(3)] for i in range(3)]), A1)
    Ab, bb = gh.evaluate(cache, k, A2, b2, bs)
    assert np.array_equal(np.block([[Ab.array[i, j] for j in range(3)] for i in range(3)]), A2)
    assert np.array_equal(np.concatenate(list(bb.array)), b2)
    with pytest.raises(ValueError):
        gh.evaluate(cache, k, A2[:-1, :-1], b2[:-1], bs)
