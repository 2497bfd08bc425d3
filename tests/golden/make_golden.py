"""Generates tests/golden/static_condensation_lapack.npz.

Golden vectors for StaticCondensationMap / BackwardStaticCondensationMap made
by an independent LAPACK (scipy.linalg.lapack, the same dgetrf/dgetrs the
reference reaches through LinearAlgebra.LAPACK) executing the reference's call
sequence literally:

  forward  (src/StaticCondensationMap.jl:179-192):
    LU, ipiv = getrf(A11); A12 = getrs(LU, ipiv, A12); A22 -= A21 A12;
    b1 = getrs(LU, ipiv, b1); b2 -= A21 b1          -> (S, g) = (A22, b2)
  backward (src/BackwardStaticCondensationMap.jl:88-99):
    b1 -= A12 x; LU, ipiv = getrf(A11); b1 = getrs(LU, ipiv, b1)  -> u

Inputs: the block structure of test/StaticCondensationMapTests.jl (3x3 blocks
of size 3, blocks [2:3,2:3] untouched, x + c offsets) with seeded random x,
plus seeded random well-conditioned blocks of the 2D/3D Darcy HDG sizes.
Run: python tests/golden/make_golden.py
"""
import os

import numpy as np
from scipy.linalg import lapack

HERE = os.path.dirname(os.path.abspath(__file__))


def forward(A, b, ni):
    A11 = A[:ni, :ni].copy(order="F")
    A12 = A[:ni, ni:].copy(order="F")
    A21 = A[ni:, :ni].copy(order="F")
    A22 = A[ni:, ni:].copy(order="F")
    b1 = b[:ni].copy()
    b2 = b[ni:].copy()
    lu, piv, info = lapack.dgetrf(A11)
    assert info == 0
    A12, info = lapack.dgetrs(lu, piv, A12)
    A22 = A22 - A21 @ A12
    b1, info = lapack.dgetrs(lu, piv, b1)
    b2 = b2 - A21 @ b1
    return A22, b2


def backward(A, b, x, ni):
    A11 = A[:ni, :ni].copy(order="F")
    A12 = A[:ni, ni:]
    b1 = b[:ni] - A12 @ x
    lu, piv, info = lapack.dgetrf(A11)
    assert info == 0
    u, info = lapack.dgetrs(lu, piv, b1)
    return u


def reference_test_case(rng):
    """test/StaticCondensationMapTests.jl:6-28 with a seeded rand."""
    x = rng.random((3, 3))
    blocks = {(0, 0): x, (1, 0): x + 1, (2, 0): x + 2, (0, 1): x + 3, (0, 2): x + 5}
    A = np.zeros((9, 9))
    for (i, j), blk in blocks.items():
        A[3 * i:3 * i + 3, 3 * j:3 * j + 3] = blk
    xv = rng.random(3)
    b = np.concatenate([xv, xv + 1, xv + 2])
    return A, b, 6


def main():
    rng = np.random.default_rng(20240601)
    cases = [reference_test_case(rng)]
    for ni, nf in [(12, 8), (27, 12), (48, 16), (108, 54)]:
        n = ni + nf
        A = rng.normal(size=(n, n))
        A[np.arange(ni), np.arange(ni)] += 2.0 * np.sqrt(n)
        cases.append((A, rng.normal(size=n), ni))
    out = {}
    for idx, (A, b, ni) in enumerate(cases):
        S, g = forward(A, b, ni)
        x = rng.normal(size=A.shape[0] - ni)
        u = backward(A, b, x, ni)
        out["A%d" % idx] = A
        out["b%d" % idx] = b
        out["ni%d" % idx] = np.array(ni)
        out["S%d" % idx] = S
        out["g%d" % idx] = g
        out["x%d" % idx] = x
        out["u%d" % idx] = u
    out["ncases"] = np.array(len(cases))
    np.savez_compressed(os.path.join(HERE, "static_condensation_lapack.npz"), **out)


if __name__ == "__main__":
    main()
