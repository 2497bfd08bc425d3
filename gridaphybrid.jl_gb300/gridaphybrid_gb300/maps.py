"""Gridap-style cell maps of GridapHybrid.jl, evaluated on the GPU.

Mirrors the Gridap.Fields.Map protocol the reference uses:

* ``return_cache(k, args...)`` -> cache, ``evaluate(cache, k, args...)`` -> value
  for one cell (a batch of one), and
* ``lazy_map(k, cell_args...)`` over all cells, which is one batched GPU call
  instead of the reference's per-cell iteration.

Maps: StaticCondensationMap (src/StaticCondensationMap.jl),
BackwardStaticCondensationMap (src/BackwardStaticCondensationMap.jl),
SumFacetsMap (src/SumFacetsMap.jl) and Scalar2ArrayBlockMap
(src/Scalar2ArrayBlockMap.jl).  ArrayBlock mirrors
Gridap.Fields.ArrayBlock (a nested array of blocks plus a ``touched`` mask).
Block bookkeeping (which blocks exist, densification into one dense array)
is host-side layout work; every arithmetic operation runs in
libgridaphybrid_gb300 on the GPU.
"""
import itertools

import numpy as np

from . import _lib


class ArrayBlock:
    """Gridap.Fields.ArrayBlock: ``array`` (object ndarray of blocks) + ``touched``."""

    def __init__(self, array, touched):
        self.array = np.asarray(array, dtype=object) if not isinstance(array, np.ndarray) else array
        self.touched = np.asarray(touched, dtype=bool)
        if self.array.shape != self.touched.shape:
            raise ValueError("array and touched must have the same shape")

    @property
    def shape(self):
        return self.touched.shape

    def __getitem__(self, idx):
        return self.array[idx]

    def __repr__(self):
        return "ArrayBlock(shape=%s, touched=%s)" % (self.shape, self.touched.tolist())


def MatrixBlock(blocks, touched):
    a = np.empty(np.shape(touched), dtype=object)
    for idx in itertools.product(*[range(s) for s in a.shape]):
        a[idx] = blocks[idx[0]][idx[1]] if touched[idx[0]][idx[1]] else None
    return ArrayBlock(a, touched)


def VectorBlock(blocks, touched):
    a = np.empty(len(touched), dtype=object)
    for i, t in enumerate(touched):
        a[i] = blocks[i] if t else None
    return ArrayBlock(a, touched)


def _check_preconditions(interior_fields, boundary_fields):
    """src/StaticCondensationMap.jl:16-34: the fields form a partition of 1:n."""
    nfields = len(interior_fields) + len(boundary_fields)
    seen = set()
    for f in list(interior_fields) + list(boundary_fields):
        if f < 1 or f > nfields or f in seen:
            return False
        seen.add(f)
    return len(seen) == nfields


def _block_sizes(A):
    """Row block sizes of a MatrixBlock (src/StaticCondensationMap.jl:72-84)."""
    nr, nc = A.shape
    brs = [None] * nr
    bcs = [None] * nc
    for i in range(nr):
        for j in range(nc):
            if A.touched[i, j]:
                blk = np.asarray(A.array[i, j])
                brs[i] = blk.shape[0]
                bcs[j] = blk.shape[1]
    if any(s is None for s in brs) or brs != bcs:
        raise ValueError("every block row/column needs a touched block and brs == bcs")
    return brs


def _densify(A, b, order, brs):
    """Dense (n x n) matrix and vector of the blocks listed in `order` (1-based);
    untouched blocks are zero (DensifyInnerMostBlockLevelMap)."""
    offs = np.cumsum([0] + [brs[f - 1] for f in order])
    n = int(offs[-1])
    Ad = np.zeros((n, n))
    bd = np.zeros(n)
    for I, fi in enumerate(order):
        if b.touched[fi - 1]:
            bd[offs[I]:offs[I + 1]] = np.asarray(b.array[fi - 1], dtype=np.float64)
        for J, fj in enumerate(order):
            if A.touched[fi - 1, fj - 1]:
                Ad[offs[I]:offs[I + 1], offs[J]:offs[J + 1]] = np.asarray(A.array[fi - 1, fj - 1])
    return Ad, bd


class StaticCondensationMap:
    """S = A_ff - A_fi A_ii^{-1} A_if, g = b_f - A_fi A_ii^{-1} b_i per cell
    (src/StaticCondensationMap.jl:3-14, evaluate! :146-196)."""

    def __init__(self, interior_fields, boundary_fields, precision=_lib.HDG_PREC_FP64, context=None):
        if not _check_preconditions(interior_fields, boundary_fields):
            raise ValueError("interior/boundary fields must partition 1:nfields")
        self.interior_fields = list(interior_fields)
        self.boundary_fields = list(boundary_fields)
        self.precision = precision
        self.ctx = context

    def _context(self):
        return self.ctx or _lib.default_context()

    def return_cache(self, A, b):
        brs = _block_sizes(A)
        ni = sum(brs[f - 1] for f in self.interior_fields)
        nf = sum(brs[f - 1] for f in self.boundary_fields)
        return {"brs": brs, "ni": ni, "nf": nf}

    def evaluate(self, cache, A, b):
        Ad, bd = self._dense(cache, A, b)
        return self._call(Ad[None], bd[None], cache["ni"], batched=False)

    def _dense(self, cache, A, b):
        return _densify(A, b, self.interior_fields + self.boundary_fields, cache["brs"])

    def condense_dense(self, Ad, bd, ni):
        """Batched condensation of dense cell blocks: Ad (ncells, n, n), bd (ncells, n)."""
        return self._call(np.asarray(Ad), np.asarray(bd), ni, batched=True)

    def _call(self, Ad, bd, ni, batched):
        ctx = self._context()
        ncells, n, _ = Ad.shape
        nf = n - ni
        Acm = np.ascontiguousarray(np.transpose(Ad, (0, 2, 1)), dtype=np.float64)  # column-major per cell
        bd = _lib.as_f64(bd)
        S = np.empty((ncells, nf, nf))
        g = np.empty((ncells, nf))
        info = np.zeros(ncells, dtype=np.int32)
        ctx.check(ctx.lib.hdg_static_condensation(ctx.handle, self.precision, ncells, ni, nf,
                                                  _lib.ptr(Acm), _lib.ptr(bd), _lib.ptr(S),
                                                  _lib.ptr(g), _lib.ptr(info)))
        S = np.transpose(S, (0, 2, 1))  # back to row-major view of the column-major result
        return (S, g) if batched else (S[0], g[0])




class BackwardStaticCondensationMap:
    """u_i = A_ii^{-1}(b_i - A_if x) per cell, re-blocked as
    [interior blocks..., skeleton blocks...]
    (src/BackwardStaticCondensationMap.jl:6-19, evaluate! :61-112, reblock :115-151)."""

    def __init__(self, interior_fields, boundary_fields, precision=_lib.HDG_PREC_FP64, context=None):
        self.static_condensation = StaticCondensationMap(interior_fields, boundary_fields, precision, context)

    def return_cache(self, A, b, x):
        return self.static_condensation.return_cache(A, b)

    def evaluate(self, cache, A, b, x):
        sc = self.static_condensation
        Ad, bd = sc._dense(cache, A, b)
        if isinstance(x, ArrayBlock):  # densify a blocked skeleton vector (:104-112)
            x = np.concatenate([np.asarray(x.array[i]) for i in range(x.shape[0]) if x.touched[i]])
        u = self.backward_dense(Ad[None], bd[None], np.asarray(x, dtype=np.float64)[None], cache["ni"])[0]
        brs = cache["brs"]
        blocks, off = [], 0
        for f in sc.interior_fields:
            blocks.append(u[off:off + brs[f - 1]])
            off += brs[f - 1]
        off = 0
        for f in sc.boundary_fields:
            blocks.append(np.asarray(x)[off:off + brs[f - 1]])
            off += brs[f - 1]
        return VectorBlock(blocks, [True] * len(blocks))

    def backward_dense(self, Ad, bd, x, ni):
        sc = self.static_condensation
        ctx = sc._context()
        ncells, n, _ = Ad.shape
        nf = n - ni
        Acm = np.ascontiguousarray(np.transpose(Ad, (0, 2, 1)), dtype=np.float64)
        bd = _lib.as_f64(bd)
        x = _lib.as_f64(x)
        u = np.empty((ncells, ni))
        info = np.zeros(ncells, dtype=np.int32)
        ctx.check(ctx.lib.hdg_backward_static_condensation(ctx.handle, sc.precision, ncells, ni, nf,
                                                           _lib.ptr(Acm), _lib.ptr(bd), _lib.ptr(x),
                                                           _lib.ptr(u), _lib.ptr(info)))
        return u


def _leaves(ab, prefix=()):
    """(path, array) leaves of a nested ArrayBlock."""
    out = []
    for idx in itertools.product(*[range(s) for s in ab.shape]):
        if not ab.touched[idx]:
            continue
        v = ab.array[idx]
        if isinstance(v, ArrayBlock):
            out.extend(_leaves(v, prefix + ((idx, ab.shape),)))
        else:
            out.append((prefix + ((idx, ab.shape),), np.asarray(v, dtype=np.float64)))
    return out


def _build_nested(leaves):
    """Rebuild a nested ArrayBlock from {path: array}."""
    shape = leaves[0][0][0][1]
    arr = np.empty(shape, dtype=object)
    touched = np.zeros(shape, dtype=bool)
    groups = {}
    for path, val in leaves:
        idx = path[0][0]
        groups.setdefault(idx, []).append((path[1:], val))
    for idx, items in groups.items():
        touched[idx] = True
        if len(items) == 1 and items[0][0] == ():
            arr[idx] = items[0][1]
        else:
            arr[idx] = _build_nested(items)
    return ArrayBlock(arr, touched)


class SumFacetsMap:
    """Sum of the per-facet blocks of a cell, folded with (+) left to right
    (src/SumFacetsMap.jl:1-30); untouched + touched = touched."""

    def __init__(self, context=None):
        self.ctx = context

    def return_cache(self, a):
        if not (isinstance(a, ArrayBlock) and a.touched.all() and a.shape[0] >= 2):
            raise ValueError("SumFacetsMap needs a fully touched VectorBlock of >= 2 facet blocks")
        return None

    def evaluate(self, cache, a):
        ctx = self.ctx or _lib.default_context()
        nfac = a.shape[0]
        per_facet = [dict(_leaves(a.array[f])) if isinstance(a.array[f], ArrayBlock)
                     else {(): np.asarray(a.array[f], dtype=np.float64)} for f in range(nfac)]
        paths = []
        for d in per_facet:
            for p in d:
                if p not in paths:
                    paths.append(p)
        shapes = {}
        for d in per_facet:
            for p, v in d.items():
                shapes[p] = v.shape
        blocks = []
        for p in paths:
            for d in per_facet:
                blocks.append(d[p].ravel() if p in d else np.zeros(int(np.prod(shapes[p]))))
        lens = [int(np.prod(shapes[p])) for p in paths]
        # one call per distinct leaf size keeps the layout rectangular
        out = {}
        for L in sorted(set(lens)):
            sel = [i for i, l in enumerate(lens) if l == L]
            stack = np.ascontiguousarray(
                np.stack([np.stack(blocks[i * nfac:(i + 1) * nfac]) for i in sel]), dtype=np.float64)
            res = np.empty((len(sel), L))
            ctx.check(ctx.lib.hdg_sum_facets(ctx.handle, len(sel), nfac, L, _lib.ptr(stack), _lib.ptr(res)))
            for j, i in enumerate(sel):
                out[paths[i]] = res[j].reshape(shapes[paths[i]])
        if paths == [()]:
            return out[()]
        return _build_nested([(p, out[p]) for p in paths])


class Scalar2ArrayBlockMap:
    """Scalar2ArrayBlockMap (src/Scalar2ArrayBlockMap.jl:1-69): a dense cell
    matrix A and vector b split into an ArrayBlock of bs[i] x bs[j] blocks and a
    vector ArrayBlock of bs[i] blocks, every block touched -- the re-blocking of
    a cell system by field (src/HybridAffineFEOperators.jl:343-356).  Layout
    work only: the blocks are copies of A's and b's sub-ranges.  Called as the
    reference calls it, with (A, b), bs or with A, b, bs."""

    @staticmethod
    def _args(args):
        if len(args) == 2:
            (A, b), bs = args
        else:
            A, b, bs = args
        return np.asarray(A), np.asarray(b), [int(x) for x in bs]

    def return_cache(self, *args):
        A, b, bs = self._args(args)
        n = len(bs)
        Ab = np.empty((n, n), dtype=object)
        bb = np.empty(n, dtype=object)
        for i in range(n):
            bb[i] = np.empty(bs[i], dtype=b.dtype)
            for j in range(n):
                Ab[i, j] = np.empty((bs[i], bs[j]), dtype=A.dtype)
        return ArrayBlock(Ab, np.ones((n, n), dtype=bool)), ArrayBlock(bb, np.ones(n, dtype=bool))

    def evaluate(self, cache, *args):
        A, b, bs = self._args(args)
        if A.shape != (sum(bs), sum(bs)) or b.shape != (sum(bs),):
            raise ValueError("A and b must be sum(bs) x sum(bs) and sum(bs)")
        Ab, bb = cache
        off = np.concatenate([[0], np.cumsum(bs)])
        for j in range(len(bs)):
            for i in range(len(bs)):
                if Ab.array[i, j].shape != (bs[i], bs[j]):
                    raise ValueError("cache blocks do not match bs")
                Ab.array[i, j][...] = A[off[i]:off[i + 1], off[j]:off[j + 1]]
        for i in range(len(bs)):
            bb.array[i][...] = b[off[i]:off[i + 1]]
        return Ab, bb


def densify(ab):
    """DensifyInnerMostBlockLevelMap for a two-level block (outer blocks whose
    entries are blocks): each outer entry becomes one dense array."""
    arr = np.empty(ab.shape, dtype=object)
    for idx in itertools.product(*[range(s) for s in ab.shape]):
        v = ab.array[idx]
        if not ab.touched[idx]:
            arr[idx] = None
            continue
        if isinstance(v, ArrayBlock):
            if v.array.ndim == 1:
                arr[idx] = np.concatenate([np.asarray(v.array[i]) for i in range(v.shape[0])])
            else:
                rows = []
                for i in range(v.shape[0]):
                    rows.append(np.hstack([np.asarray(v.array[i, j]) for j in range(v.shape[1])]))
                arr[idx] = np.vstack(rows)
        else:
            arr[idx] = v
    return ArrayBlock(arr, ab.touched.copy())


def return_cache(k, *args):
    return k.return_cache(*args)


def evaluate(cache, k, *args):
    return k.evaluate(cache, *args)


def lazy_map(k, *cell_args):
    """Apply a map to every cell.  For the condensation maps the cells are
    densified once and processed in one batched GPU call."""
    if isinstance(k, StaticCondensationMap):
        A_cells, b_cells = cell_args
        cache = k.return_cache(A_cells[0], b_cells[0])
        dense = [k._dense(cache, A, b) for A, b in zip(A_cells, b_cells)]
        Ad = np.stack([d[0] for d in dense])
        bd = np.stack([d[1] for d in dense])
        S, g = k._call(Ad, bd, cache["ni"], batched=True)
        return list(zip(S, g))
    if isinstance(k, BackwardStaticCondensationMap):
        A_cells, b_cells, x_cells = cell_args
        sc = k.static_condensation
        cache = sc.return_cache(A_cells[0], b_cells[0])
        dense = [sc._dense(cache, A, b) for A, b in zip(A_cells, b_cells)]
        Ad = np.stack([d[0] for d in dense])
        bd = np.stack([d[1] for d in dense])
        u = k.backward_dense(Ad, bd, np.stack([np.asarray(x, dtype=np.float64) for x in x_cells]), cache["ni"])
        return list(u)
    return [k.evaluate(k.return_cache(*args), *args) for args in zip(*cell_args)]
