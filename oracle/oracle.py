"""TEST INFRASTRUCTURE ONLY — ctypes wrapper of the oracle (rcb_oracle.cpp).

The oracle is a CPU restatement of coupe's Rcb / Rib used by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.  The
product never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "build", "liboracle_rcb.so")

REF32, F64 = 0, 1
NAN_RIGHT = 0x100  # mode flag: NaN keys always go right (the GPU rule)
FSUM_SEQ, FSUM_FIXED = 0, 1
_WT = {np.dtype(np.int32): 0, np.dtype(np.int64): 1, np.dtype(np.float64): 2}


class Stats(ctypes.Structure):
    _fields_ = [("splits", ctypes.c_uint64), ("iterations", ctypes.c_uint64),
                ("max_iterations", ctypes.c_uint64), ("pivot_ties", ctypes.c_uint64),
                ("active_points", ctypes.c_uint64), ("root_sum", ctypes.c_double),
                ("fixed_scale", ctypes.c_int), ("pad", ctypes.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "pad"}


_lib = None


def build():
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(PATH):
            build()
        L = ctypes.CDLL(PATH)
        vp, u64, i32, dbl = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.c_double
        L.oracle_rcb.argtypes = [vp, u64, i32, vp, i32, vp, u64, dbl, i32, i32, i32, ctypes.POINTER(Stats)]
        L.oracle_rcb.restype = i32
        L.oracle_rib.argtypes = [vp, u64, i32, vp, i32, vp, u64, dbl, i32, i32, i32, vp, ctypes.POINTER(Stats)]
        L.oracle_rib.restype = i32
        L.oracle_record_splits.argtypes = [vp, u64]
        L.oracle_record_splits.restype = None
        L.oracle_rib_matrix.argtypes = [u64, i32, vp, vp]
        L.oracle_rib_matrix_weighted.argtypes = [u64, i32, vp, vp, vp]
        L.oracle_rib_matrix_weighted.restype = i32
        L.oracle_rib_matrix.restype = i32
        L.oracle_map_points.argtypes = [vp, u64, i32, vp, vp]
        L.oracle_bbox.argtypes = [vp, u64, i32, vp, vp]
        L.oracle_inertia_matrix.argtypes = [vp, u64, i32, vp]
        L.oracle_inertia_vector.argtypes = [vp, i32, vp]
        L.oracle_householder.argtypes = [vp, i32, vp]
        L.oracle_fixed_scale.argtypes = [vp, u64]
        L.oracle_fixed_scale.restype = i32
        L.oracle_fixed_sum.argtypes = [vp, u64, i32]
        L.oracle_fixed_sum.restype = dbl
        L.oracle_split_f32_u32.argtypes = [vp, vp, u64, dbl, ctypes.c_float, ctypes.c_float, vp, vp]
        L.oracle_split_f32_u32.restype = u64
        L.oracle_reorder_split_f32.argtypes = [vp, u64, u64]
        L.oracle_reorder_split_f32.restype = u64
        _lib = L
    return _lib


def _prep(points, weights):
    p = np.ascontiguousarray(np.asarray(points, dtype=np.float64))
    w = np.asarray(weights)
    if w.dtype.kind in "iu" and w.dtype != np.int32:
        w = w.astype(np.int64)
    elif w.dtype.kind == "f":
        w = w.astype(np.float64)
    return p, np.ascontiguousarray(w)


class _SplitRecorder:
    """Records the split position of every tree node (heap id) of one call."""

    def __init__(self, iter_count):
        self.buf = np.full((1 << (iter_count + 1)) - 1 if iter_count < 30 else 1, np.nan)

    def __enter__(self):
        lib().oracle_record_splits(self.buf.ctypes.data, len(self.buf))
        return self.buf

    def __exit__(self, *a):
        lib().oracle_record_splits(None, 0)


def rcb(points, weights, iter_count, tolerance, mode=REF32, fsum=FSUM_FIXED, threads=1, splits=False):
    """Part ids (uint64) of coupe's Rcb, and run statistics; with splits=True
    the statistics also hold "split_pos": the position of each node's split
    by heap id (NaN where no split was made)."""
    p, w = _prep(points, weights)
    n, dim = p.shape
    out = np.zeros(n, dtype=np.uint64)
    st = Stats()
    rec = _SplitRecorder(iter_count) if splits else None
    if rec:
        rec.__enter__()
    try:
        rc = lib().oracle_rcb(out.ctypes.data, n, dim, p.ctypes.data, _WT[w.dtype], w.ctypes.data,
                              iter_count, tolerance, mode, fsum, threads, ctypes.byref(st))
    finally:
        if rec:
            rec.__exit__()
    if rc != 0:
        raise ValueError("oracle_rcb failed (%d)" % rc)
    d = st.as_dict()
    if rec:
        d["split_pos"] = rec.buf
    return out, d


def rcb_sets(points, weights, set_offsets, iter_counts, tolerance, mode=REF32, fsum=FSUM_FIXED, threads=1):
    """Part ids of independent Rcb runs, one per set (rows set_offsets[k]:
    set_offsets[k + 1], iter_counts[k]); each set's ids start at 0."""
    p, w = _prep(points, weights)
    out = np.zeros(len(p), dtype=np.uint64)
    for k, it in enumerate(iter_counts):
        a, b = int(set_offsets[k]), int(set_offsets[k + 1])
        if b > a:
            out[a:b], _ = rcb(p[a:b], w[a:b], int(it), tolerance, mode=mode, fsum=fsum, threads=threads)
    return out


def rib(points, weights, iter_count, tolerance, mode=REF32, fsum=FSUM_FIXED, threads=1, matrix=None,
        splits=False):
    p, w = _prep(points, weights)
    n, dim = p.shape
    out = np.zeros(n, dtype=np.uint64)
    st = Stats()
    m = None if matrix is None else np.ascontiguousarray(np.asarray(matrix, dtype=np.float64))
    rec = _SplitRecorder(iter_count) if splits else None
    if rec:
        rec.__enter__()
    try:
        rc = lib().oracle_rib(out.ctypes.data, n, dim, p.ctypes.data, _WT[w.dtype], w.ctypes.data,
                              iter_count, tolerance, mode, fsum, threads,
                              m.ctypes.data if m is not None else None, ctypes.byref(st))
    finally:
        if rec:
            rec.__exit__()
    if rc != 0:
        raise ValueError("oracle_rib failed (%d)" % rc)
    d = st.as_dict()
    if rec:
        d["split_pos"] = rec.buf
    return out, d


def rib_matrix(points):
    p = np.ascontiguousarray(np.asarray(points, dtype=np.float64))
    n, dim = p.shape
    m = np.zeros((dim, dim))
    rc = lib().oracle_rib_matrix(n, dim, p.ctypes.data, m.ctypes.data)
    if rc != 0:
        raise ValueError("oracle_rib_matrix failed (%d)" % rc)
    return m


def rib_matrix_weighted(points, weights):
    """The basis change of the weighted inertia matrix (the GPU library's
    opt-in; coupe's own is unweighted)."""
    p = np.ascontiguousarray(np.asarray(points, dtype=np.float64))
    w = np.ascontiguousarray(np.asarray(weights, dtype=np.float64))
    n, dim = p.shape
    m = np.zeros((dim, dim))
    rc = lib().oracle_rib_matrix_weighted(n, dim, p.ctypes.data, w.ctypes.data, m.ctypes.data)
    if rc != 0:
        raise ValueError("oracle_rib_matrix_weighted failed (%d)" % rc)
    return m


def map_points(points, matrix):
    p = np.ascontiguousarray(np.asarray(points, dtype=np.float64))
    n, dim = p.shape
    m = np.ascontiguousarray(np.asarray(matrix, dtype=np.float64))
    out = np.zeros_like(p)
    lib().oracle_map_points(p.ctypes.data, n, dim, m.ctypes.data, out.ctypes.data)
    return out


def bbox(points):
    p = np.ascontiguousarray(np.asarray(points, dtype=np.float64))
    n, dim = p.shape
    lo, hi = np.zeros(dim), np.zeros(dim)
    lib().oracle_bbox(p.ctypes.data, n, dim, lo.ctypes.data, hi.ctypes.data)
    return lo, hi


def inertia_matrix(points):
    p = np.ascontiguousarray(np.asarray(points, dtype=np.float64))
    n, dim = p.shape
    m = np.zeros((dim, dim))
    lib().oracle_inertia_matrix(p.ctypes.data, n, dim, m.ctypes.data)
    return m


def inertia_vector(m):
    m = np.ascontiguousarray(np.asarray(m, dtype=np.float64))
    dim = m.shape[0]
    v = np.zeros(dim)
    lib().oracle_inertia_vector(m.ctypes.data, dim, v.ctypes.data)
    return v


def householder(v):
    v = np.ascontiguousarray(np.asarray(v, dtype=np.float64))
    dim = v.shape[0]
    h = np.zeros((dim, dim))
    lib().oracle_householder(v.ctypes.data, dim, h.ctypes.data)
    return h


def fixed_scale(w):
    w = np.ascontiguousarray(np.asarray(w, dtype=np.float64))
    return lib().oracle_fixed_scale(w.ctypes.data, len(w))


def fixed_sum(w, s):
    w = np.ascontiguousarray(np.asarray(w, dtype=np.float64))
    return lib().oracle_fixed_sum(w.ctypes.data, len(w), s)


def split_f32_u32(keys, weights, tolerance, mn, mx):
    """One par_rcb_split on 1-D keys; returns (left keys, right keys,
    left weights, right weights, weight_left, split_pos)."""
    k = np.ascontiguousarray(np.asarray(keys, dtype=np.float32)).copy()
    w = np.ascontiguousarray(np.asarray(weights, dtype=np.uint32)).copy()
    wl = ctypes.c_uint32()
    sp = ctypes.c_float()
    nl = lib().oracle_split_f32_u32(k.ctypes.data, w.ctypes.data, len(k), tolerance, mn, mx,
                                    ctypes.byref(wl), ctypes.byref(sp))
    return k[:nl], k[nl:], w[:nl], w[nl:], wl.value, sp.value


def reorder_split_f32(keys, pivot_index):
    k = np.ascontiguousarray(np.asarray(keys, dtype=np.float32)).copy()
    nl = lib().oracle_reorder_split_f32(k.ctypes.data, len(k), pivot_index)
    return k[:nl], k[nl:]


# ---------------------------------------------------------------------------
# coupe::imbalance (coupe/src/imbalance.rs), restated on the host.
# ---------------------------------------------------------------------------
def parts_load(partition, num_parts, weights):
    """compute_parts_load (imbalance.rs:14-39): the sum of the weights of
    each part.  Integer loads wrap around in the weights' type (coupe's
    release build); f64 loads are this oracle's fixed-point sums (one scale
    for all n weights, fixed_scale / fixed_sum), the order-independent form
    the GPU computes.  A part id >= num_parts raises IndexError (coupe's
    `acc[part]` panics)."""
    ids = np.asarray(partition, dtype=np.uint64)
    w = np.asarray(weights)
    if len(ids) != len(w):
        raise ValueError("partition and weights differ in length")
    if len(ids) and int(ids.max()) >= num_parts:
        raise IndexError("part id out of range")
    if w.dtype == np.float64:
        s = fixed_scale(w)
        order = np.argsort(ids, kind="stable")
        ws = w[order]
        bounds = np.searchsorted(ids[order], np.arange(num_parts + 1, dtype=np.uint64))
        return np.array([fixed_sum(ws[bounds[p]:bounds[p + 1]], s) for p in range(num_parts)], dtype=np.float64)
    acc = np.zeros(num_parts, dtype=np.int64)
    np.add.at(acc, ids.astype(np.int64), w.astype(np.int64))  # wraps mod 2^64
    return acc.astype(w.dtype) if w.dtype == np.int32 else acc


def imbalance(num_parts, partition, weights):
    """imbalance (imbalance.rs:41-77): 0 without parts (before any load is
    computed); else the total load summed in the weights' type, the ideal
    total / num_parts in f64, 0 when that is 0, and the largest
    (load - ideal) / ideal."""
    if num_parts == 0:
        return 0.0
    loads = parts_load(partition, num_parts, weights)
    if loads.dtype == np.float64:
        total = 0.0
        for v in loads:
            total += float(v)
    else:
        with np.errstate(over="ignore"):
            total = float(np.sum(loads, dtype=loads.dtype))
    ideal = total / float(num_parts)
    if ideal == 0.0:
        return 0.0
    return max((float(v) - ideal) / ideal for v in loads)


def barycentres(coords, nodes):
    """mesh-part's points (tools/lib/lib.rs:511-539) for one element block:
    per element, 0.0 plus its node coordinates in node order, divided by the
    node count."""
    c = np.asarray(coords, dtype=np.float64)
    v = np.asarray(nodes, dtype=np.int64)
    acc = np.zeros((len(v), c.shape[1]))
    for j in range(v.shape[1]):
        acc = acc + c[v[:, j]]
    return acc / float(v.shape[1])


# ---------------------------------------------------------------------------
# coupe::Grid::rcb (coupe/src/cartesian/mod.rs:130-179, cartesian/rcb.rs:52-281)
# restated on the host.  The weighted median replays rayon's fold_chunks with
# `threads` workers (cartesian/rcb.rs:67-72), so the split positions depend
# on that count exactly as coupe's do.  The root's f64 total is the
# fixed-point sum rounded once (coupe's rayon sum has no fixed order).
# ---------------------------------------------------------------------------
GRID_TOLERANCE = 0.01  # cartesian/rcb.rs:45

_INT_RANGE = {np.dtype(np.int32): (-(2**31), 2**31 - 1), np.dtype(np.int64): (-(2**63), 2**63 - 1)}


def _w_from_f64(x, dt):
    """f64 `as` W: truncation toward zero, saturating, NaN -> 0."""
    if dt == np.float64:
        return float(x)
    if x != x:
        return 0
    lo, hi = _INT_RANGE[dt]
    if x >= hi:
        return hi
    if x <= lo:
        return lo
    return int(x)


def _w_wrap(v, dt):
    if dt == np.float64:
        return float(v)
    bits = 32 if dt == np.int32 else 64
    v &= (1 << bits) - 1
    return v - (1 << bits) if v >> (bits - 1) else v


def grid_weighted_median(weights, total, threads, dt):
    """weighted_median (cartesian/rcb.rs:53-101): (position, left weight).
    threads >= 2 (with one worker coupe's loop does not end)."""
    dt = np.dtype(dt)
    ideal = float(total) / 2.0
    min_part = _w_from_f64(ideal * (1.0 - GRID_TOLERANCE), dt)
    max_part = _w_from_f64(ideal * (1.0 + GRID_TOLERANCE), dt)
    zero = 0.0 if dt == np.float64 else 0
    w = [float(x) if dt == np.float64 else int(x) for x in weights]
    lo, hi, left = 0, len(w), zero
    while True:
        cs = max(1, (hi - lo) // threads)
        left0, prefix = left, zero
        for start in range(lo, hi, cs):
            pcw = _w_wrap(left0 + prefix, dt)
            csum = zero
            for x in w[start:min(start + cs, hi)]:
                csum = _w_wrap(csum + x, dt)
            prefix = _w_wrap(prefix + csum, dt)
            if pcw < min_part:
                lo, left = start, pcw
            elif max_part < pcw:
                hi = start
                break
            else:
                return start, pcw
        if lo + 1 >= hi:
            return lo, left


def _grid_axis_sums(w, off, sz, coord, dt):
    """The sums of the subgrid's slabs along `coord`, each in coupe's order
    (cartesian/rcb.rs:119-141, 192-238): 2D w[y, x]; 3D w[z, y, x]."""
    D = w.ndim
    out = []
    rng = [range(off[d], off[d] + sz[d]) for d in range(D)]
    for p in rng[coord]:
        if D == 2:
            x0, x1, y0, y1 = off[0], off[0] + sz[0], off[1], off[1] + sz[1]
            slab = w[y0:y1, p] if coord == 0 else w[p, x0:x1]
        else:
            x0, x1, y0, y1, z0, z1 = (off[0], off[0] + sz[0], off[1], off[1] + sz[1], off[2], off[2] + sz[2])
            if coord == 0:
                slab = w[z0:z1, y0:y1, p].T  # y outer, z inner
            elif coord == 1:
                slab = w[z0:z1, p, x0:x1]  # z outer, x inner
            else:
                slab = w[p, y0:y1, x0:x1].T  # x outer, y inner
        flat = np.ascontiguousarray(slab).reshape(-1)
        if dt == np.float64:
            out.append(float(np.cumsum(flat)[-1]) if len(flat) else 0.0)
        else:
            out.append(_w_wrap(int(flat.astype(np.int64).sum(dtype=np.int64)), dt))
    return out


def grid_rcb(size, weights, iter_count, threads):
    """Grid::rcb (cartesian/mod.rs:130-179): part ids of the cells (index
    x + width * (y + height * z)), in [0, 2^iter_count)."""
    D = len(size)
    wv = np.asarray(weights)
    dt = wv.dtype
    w = wv.reshape(tuple(reversed(size)))
    if dt == np.float64:
        total = fixed_sum(wv, fixed_scale(wv)) if len(wv) else 0.0
    else:
        total = _w_wrap(int(wv.astype(np.int64).sum(dtype=np.int64)), dt)
    tree = {}

    def rec(node, off, sz, tot, iters, coord):
        if sz[coord] == 0 or iters == 0:
            tree[node] = None
            return
        axis = _grid_axis_sums(w, off, sz, coord, dt)
        pos, left = grid_weighted_median(axis, tot, threads, dt)
        at = pos + off[coord]
        right = _w_wrap(tot - left, dt)
        lo_sz, hi_sz, hi_off = list(sz), list(sz), list(off)
        lo_sz[coord] = at - off[coord]
        hi_sz[coord] -= at - off[coord]
        hi_off[coord] = at
        tree[node] = at
        nxt = (coord + 1) % D
        rec(2 * node + 1, off, lo_sz, left, iters - 1, nxt)
        rec(2 * node + 2, hi_off, hi_sz, right, iters - 1, nxt)

    rec(0, [0] * D, list(size), total, iter_count, 1)
    n = int(np.prod(size))
    idx = np.arange(n)
    pos = [idx % size[0], (idx // size[0]) % size[1]] + ([idx // size[0] // size[1]] if D == 3 else [])
    ids = np.zeros(n, dtype=np.uint64)
    node = np.zeros(n, dtype=np.int64)
    coord = 1
    active = np.ones(n, dtype=bool)
    while active.any():
        nxt_node = node.copy()
        for nd in np.unique(node[active]):
            at = tree.get(int(nd))
            m = active & (node == nd)
            if at is None:
                active &= ~m
                continue
            right = m & (pos[coord] >= at)
            left = m & ~right
            ids[left] = ids[left] * 2
            ids[right] = ids[right] * 2 + 1
            nxt_node[left] = 2 * nd + 1
            nxt_node[right] = 2 * nd + 2
        node = nxt_node
        coord = (coord + 1) % D
    return ids
