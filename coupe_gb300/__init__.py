"""coupe_gb300 — coupe's Rcb and Rib on a GB300 GPU.

Python mirror of coupe's partitioning interface for these two algorithms
(coupe/src/lib.rs:76-91 `Partition`, coupe/src/algorithms/recursive_bisection.rs
:780-812 `Rcb` and :902-930 `Rib`), calling the C ABI of libcoupe_gpu.so
(include/coupe.h, include/coupe_gpu.h) through ctypes.  There is no CPU
fallback: every call runs the CUDA engine, and loading fails loudly when the
library has not been built.

    import numpy as np, coupe_gb300 as coupe
    ids = np.zeros(len(points), dtype=np.uint64)
    coupe.Rcb(iter_count=10, tolerance=0.01).partition(ids, (points, weights))
"""
import ctypes
import os
from dataclasses import dataclass

import numpy as np

__all__ = [
    "Rcb", "Rib", "CoupeError", "lib", "library_path", "MODES", "last_stats",
    "rcb_device", "rib_device", "rib_matrix_device", "rcb_batched_device", "autotune_device",
    "MultiJagged", "multi_jagged_device", "axis_sort_device",
]

_HERE = os.path.dirname(os.path.abspath(__file__))
library_path = os.path.join(_HERE, "libcoupe_gpu.so")

# enum coupe_err / coupe_type / coupe_gpu_mode (include/coupe.h, coupe_gpu.h)
ERR_OK, ERR_ALLOC, ERR_CRASH, ERR_BAD_DIMENSION, ERR_BAD_TYPE, ERR_BIPART_ONLY, \
    ERR_LEN_MISMATCH, ERR_NOT_FOUND, ERR_NEG_VALUES = range(9)
COUPE_INT, COUPE_INT64, COUPE_DOUBLE = 0, 1, 2
MODES = {"ref32": 0, "f64": 1, "f32key_f64band": 2}
WEIGHTED_INERTIA = 0x100  # COUPE_GPU_WEIGHTED_INERTIA (include/coupe_gpu.h): opt-in, Rib only

# Symbols the library exports (checked by the CPU test-suite).
EXPORTED = [
    "coupe_strerror", "coupe_data_free", "coupe_data_array", "coupe_data_constant",
    "coupe_data_fn", "coupe_rcb", "coupe_rib",
    "coupe_gpu_rcb", "coupe_gpu_rib", "coupe_gpu_rcb_device", "coupe_gpu_rib_device",
    "coupe_gpu_rib_matrix", "coupe_gpu_rib_matrix_weighted", "coupe_gpu_last_stats", "coupe_gpu_last_error", "coupe_gpu_version",
    "coupe_gpu_profile", "coupe_gpu_profile_read", "coupe_gpu_kernel_name",
    "coupe_gpu_set_option", "coupe_gpu_get_option", "coupe_gpu_f64_to_f32",
    "coupe_gpu_split_noalloc", "coupe_gpu_rcb_batched", "coupe_gpu_autotune",
    "coupe_gpu_parts_load", "coupe_gpu_imbalance", "coupe_gpu_parts_load_device", "coupe_gpu_imbalance_device",
    "coupe_gpu_barycentres", "coupe_gpu_grid_rcb", "coupe_gpu_grid_rcb_device",
    "coupe_gpu_axis_sort_device", "coupe_gpu_multi_jagged", "coupe_gpu_multi_jagged_device",
]


class CoupeError(RuntimeError):
    def __init__(self, code, detail=""):
        self.code = code
        msg = lib().coupe_strerror(code).decode()
        if detail:
            msg += " (" + detail + ")"
        super().__init__(msg)


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "points", "levels", "splits", "split_steps", "max_split_steps", "hist_passes",
        "hist_points", "band_points", "kernel_launches", "algo_bytes")] + [
        ("root_weight_sum", ctypes.c_double), ("device_ms", ctypes.c_double),
        ("fixed_scale", ctypes.c_int), ("mode", ctypes.c_int), ("weight_rechecks", ctypes.c_uint64),
        ("weight_sum_error_bound", ctypes.c_double), ("host_syncs", ctypes.c_uint64)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Tuning(ctypes.Structure):
    _fields_ = [("max_nbk", ctypes.c_int), ("hist_ctas_per_sm", ctypes.c_int),
                ("reorder_chunks_per_cta", ctypes.c_int), ("hist_waves", ctypes.c_int),
                ("device_ms", ctypes.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


I_TH = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t)
_lib = None


def lib():
    """Loads libcoupe_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(library_path):
        raise ImportError("libcoupe_gpu.so not built: run `python coupe_gb300/build.py` "
                          "or __graft_entry__.build()")
    L = ctypes.CDLL(library_path)
    vp, u64, dbl, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double, ctypes.c_int
    L.coupe_strerror.argtypes = [i32]
    L.coupe_strerror.restype = ctypes.c_char_p
    L.coupe_data_free.argtypes = [vp]
    L.coupe_data_free.restype = None
    L.coupe_data_array.argtypes = [u64, i32, vp]
    L.coupe_data_array.restype = vp
    L.coupe_data_constant.argtypes = [u64, i32, vp]
    L.coupe_data_constant.restype = vp
    L.coupe_data_fn.argtypes = [vp, u64, i32, I_TH]
    L.coupe_data_fn.restype = vp
    for f in (L.coupe_rcb, L.coupe_rib):
        f.argtypes = [vp, u64, vp, vp, u64, dbl]
        f.restype = i32
    for f in (L.coupe_gpu_rcb, L.coupe_gpu_rib):
        f.argtypes = [vp, u64, vp, vp, u64, dbl, i32]
        f.restype = i32
    L.coupe_gpu_rcb_device.argtypes = [vp, u64, u64, vp, i32, vp, u64, dbl, i32, vp, vp]
    L.coupe_gpu_rcb_device.restype = i32
    L.coupe_gpu_rib_device.argtypes = [vp, u64, u64, vp, i32, vp, u64, dbl, i32, vp]
    L.coupe_gpu_rib_device.restype = i32
    L.coupe_gpu_rcb_batched.argtypes = [vp, u64, vp, u64, vp, i32, vp, vp, dbl, i32, vp]
    L.coupe_gpu_rcb_batched.restype = i32
    L.coupe_gpu_autotune.argtypes = [vp, u64, vp, u64, vp, i32, vp, vp, dbl, i32, vp, i32, ctypes.POINTER(Tuning)]
    L.coupe_gpu_autotune.restype = i32
    L.coupe_gpu_rib_matrix.argtypes = [u64, u64, vp, vp, vp]
    L.coupe_gpu_rib_matrix.restype = i32
    L.coupe_gpu_rib_matrix_weighted.argtypes = [u64, u64, vp, i32, vp, vp, vp]
    L.coupe_gpu_rib_matrix_weighted.restype = i32
    L.coupe_gpu_last_stats.argtypes = [ctypes.POINTER(Stats)]
    L.coupe_gpu_last_stats.restype = None
    L.coupe_gpu_last_error.argtypes = []
    L.coupe_gpu_last_error.restype = ctypes.c_char_p
    L.coupe_gpu_version.argtypes = []
    L.coupe_gpu_version.restype = ctypes.c_char_p
    L.coupe_gpu_profile.argtypes = [i32]
    L.coupe_gpu_profile.restype = i32
    L.coupe_gpu_profile_read.argtypes = [vp, vp, vp, i32]
    L.coupe_gpu_profile_read.restype = i32
    L.coupe_gpu_kernel_name.argtypes = [i32]
    L.coupe_gpu_kernel_name.restype = ctypes.c_char_p
    L.coupe_gpu_f64_to_f32.argtypes = [vp, vp, u64, vp]
    L.coupe_gpu_f64_to_f32.restype = i32
    L.coupe_gpu_parts_load.argtypes = [vp, u64, vp, vp]
    L.coupe_gpu_parts_load.restype = i32
    L.coupe_gpu_imbalance.argtypes = [u64, vp, vp, ctypes.POINTER(dbl)]
    L.coupe_gpu_imbalance.restype = i32
    L.coupe_gpu_parts_load_device.argtypes = [vp, u64, i32, vp, u64, vp, vp]
    L.coupe_gpu_parts_load_device.restype = i32
    L.coupe_gpu_imbalance_device.argtypes = [u64, vp, u64, i32, vp, ctypes.POINTER(dbl), vp]
    L.coupe_gpu_imbalance_device.restype = i32
    L.coupe_gpu_grid_rcb.argtypes = [vp, u64, vp, vp, u64, u64]
    L.coupe_gpu_grid_rcb.restype = i32
    L.coupe_gpu_grid_rcb_device.argtypes = [vp, u64, vp, i32, vp, u64, u64, vp]
    L.coupe_gpu_grid_rcb_device.restype = i32
    L.coupe_gpu_barycentres.argtypes = [u64, u64, vp, u64, u64, vp, vp, vp]
    L.coupe_gpu_axis_sort_device.argtypes = [vp, u64, u64, vp, u64, vp]
    L.coupe_gpu_axis_sort_device.restype = i32
    L.coupe_gpu_multi_jagged.argtypes = [vp, u64, vp, vp, u64, u64]
    L.coupe_gpu_multi_jagged.restype = i32
    L.coupe_gpu_multi_jagged_device.argtypes = [vp, u64, u64, vp, vp, u64, u64, vp]
    L.coupe_gpu_multi_jagged_device.restype = i32
    L.coupe_gpu_barycentres.restype = i32
    L.coupe_gpu_set_option.argtypes = [ctypes.c_char_p, ctypes.c_int64]
    L.coupe_gpu_set_option.restype = i32
    L.coupe_gpu_get_option.argtypes = [ctypes.c_char_p]
    L.coupe_gpu_get_option.restype = ctypes.c_int64
    _lib = L
    return L


def set_option(name, value):
    """Sets a scheduling knob (see include/coupe_gpu.h); never changes results."""
    _check(lib().coupe_gpu_set_option(name.encode(), int(value)))


def get_option(name):
    return int(lib().coupe_gpu_get_option(name.encode()))


def profile(enable=True):
    """Turns the per-launch CUDA-event profiler on or off (resets totals)."""
    _check(lib().coupe_gpu_profile(1 if enable else 0))


def profile_read():
    """{kernel: {"launches", "bytes", "ms"}} accumulated since profile()."""
    L = lib()
    cap = 64
    c = (ctypes.c_uint64 * cap)()
    b = (ctypes.c_uint64 * cap)()
    m = (ctypes.c_double * cap)()
    k = L.coupe_gpu_profile_read(c, b, m, cap)
    out = {}
    for i in range(min(k, cap)):
        if c[i]:
            out[L.coupe_gpu_kernel_name(i).decode()] = {"launches": int(c[i]), "bytes": int(b[i]), "ms": float(m[i])}
    return out


def last_stats():
    s = Stats()
    lib().coupe_gpu_last_stats(ctypes.byref(s))
    return s.as_dict()


def _check(rc):
    if rc != ERR_OK:
        raise CoupeError(rc, lib().coupe_gpu_last_error().decode())


def _weight_type(w):
    if w.dtype == np.int32:
        return COUPE_INT
    if w.dtype == np.int64:
        return COUPE_INT64
    if w.dtype == np.float64:
        return COUPE_DOUBLE
    raise TypeError("weights must be int32, int64 or float64, got %s" % w.dtype)


def _as_weights(weights, n):
    if np.isscalar(weights):
        weights = np.full(n, weights)
    w = np.asarray(weights)
    # no copy when the caller's array already has a supported type (a copy
    # would also leave pinned memory for pageable memory)
    if w.dtype.kind in "iu" and w.dtype != np.int32:
        w = w.astype(np.int64, copy=False)
    elif w.dtype.kind == "f":
        w = w.astype(np.float64, copy=False)
    return np.ascontiguousarray(w)


@dataclass
class _Bisection:
    iter_count: int = 0
    tolerance: float = 0.0
    mode: str = "ref32"
    weighted_inertia: bool = False  # Rib only: weigh the inertia matrix by the weights (not coupe's default)
    _rib = False

    def partition(self, part_ids, data):
        """Writes one part id per point into `part_ids` (uint64, length N).

        data = (points, weights): points is an (N, D) array of float64 with
        D in {2, 3}; weights an array of N int32/int64/float64 values (a
        scalar is repeated).  Mirrors Partition::partition.
        """
        points, weights = data
        p = np.ascontiguousarray(np.asarray(points, dtype=np.float64))
        if p.ndim != 2:
            raise ValueError("points must be an (N, D) array")
        n, dim = p.shape
        w = _as_weights(weights, n)
        if part_ids.dtype != np.uint64 or not part_ids.flags.c_contiguous:
            raise TypeError("part_ids must be a contiguous uint64 array")
        if len(part_ids) != n:
            raise CoupeError(ERR_LEN_MISMATCH)
        L = lib()
        dp = L.coupe_data_array(n, COUPE_DOUBLE, p.ctypes.data)
        dw = L.coupe_data_array(len(w), _weight_type(w), w.ctypes.data)
        try:
            fn = L.coupe_gpu_rib if self._rib else L.coupe_gpu_rcb
            mode = MODES[self.mode] | (WEIGHTED_INERTIA if self._rib and self.weighted_inertia else 0)
            rc = fn(part_ids.ctypes.data, dim, dp, dw, self.iter_count, self.tolerance, mode)
        finally:
            L.coupe_data_free(dp)
            L.coupe_data_free(dw)
        _check(rc)


class Rcb(_Bisection):
    """Recursive coordinate bisection (coupe::Rcb): at most 2**iter_count parts."""


class Rib(_Bisection):
    """Recursive inertial bisection (coupe::Rib): Rcb after aligning the first
    axis with the points' principal inertia axis."""
    _rib = True


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def rcb_device(part_ids, points, weights, iter_count, tolerance, mode="ref32", matrix=None, stream=None):
    """Rcb on CUDA tensors (torch): part_ids int64/uint64 (N,), points float64
    (N, D) contiguous, weights int32/int64/float64 (N,).  `matrix` (D x D)
    applies p -> matrix @ p first.  Synchronises the stream before returning."""
    import torch
    n, dim = points.shape
    wt = {torch.int32: COUPE_INT, torch.int64: COUPE_INT64, torch.float64: COUPE_DOUBLE}[weights.dtype]
    m = None
    if matrix is not None:
        m = np.ascontiguousarray(np.asarray(matrix, dtype=np.float64).reshape(dim, dim))
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    rc = lib().coupe_gpu_rcb_device(_ptr(part_ids), n, dim, _ptr(points), wt, _ptr(weights), iter_count,
                                    tolerance, MODES[mode], m.ctypes.data if m is not None else None,
                                    ctypes.c_void_p(s))
    _check(rc)


def rcb_batched_device(part_ids, points, weights, set_offsets, iter_counts, tolerance, mode="ref32", stream=None):
    """Rcb of several independent point sets in one run, on CUDA tensors:
    set k is rows set_offsets[k]:set_offsets[k + 1] of points (N, D) float64,
    weights (N,) and part_ids (N,), split into at most 2**iter_counts[k]
    parts with ids from 0, as a separate rcb_device call on that set gives.
    set_offsets (nsets + 1) and iter_counts (nsets) are host sequences."""
    import torch
    n, dim = points.shape
    wt = {torch.int32: COUPE_INT, torch.int64: COUPE_INT64, torch.float64: COUPE_DOUBLE}[weights.dtype]
    off = np.ascontiguousarray(np.asarray(set_offsets, dtype=np.uint64))
    it = np.ascontiguousarray(np.asarray(iter_counts, dtype=np.uint32))
    if off.ndim != 1 or it.ndim != 1 or len(off) != len(it) + 1:
        raise ValueError("set_offsets needs one entry more than iter_counts")
    if len(it) and int(off[-1]) != n:
        raise CoupeError(ERR_LEN_MISMATCH, "the last set offset must equal the number of points")
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    rc = lib().coupe_gpu_rcb_batched(_ptr(part_ids), len(it), off.ctypes.data, dim, _ptr(points), wt,
                                     _ptr(weights), it.ctypes.data, tolerance, MODES[mode], ctypes.c_void_p(s))
    _check(rc)


def autotune_device(part_ids, points, weights, set_offsets, iter_counts, tolerance, mode="ref32", repeats=2,
                    stream=None):
    """Times the batched call (arguments of rcb_batched_device) under each
    candidate schedule and keeps the fastest process-wide; returns it as a
    dict (max_nbk, hist_ctas_per_sm, reorder_chunks_per_cta, device_ms).
    The ids never depend on the schedule."""
    import torch
    n, dim = points.shape
    wt = {torch.int32: COUPE_INT, torch.int64: COUPE_INT64, torch.float64: COUPE_DOUBLE}[weights.dtype]
    off = np.ascontiguousarray(np.asarray(set_offsets, dtype=np.uint64))
    it = np.ascontiguousarray(np.asarray(iter_counts, dtype=np.uint32))
    if off.ndim != 1 or it.ndim != 1 or len(off) != len(it) + 1 or int(off[-1]) != n:
        raise ValueError("set_offsets must have len(iter_counts) + 1 entries ending at the number of points")
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    best = Tuning()
    rc = lib().coupe_gpu_autotune(_ptr(part_ids), len(it), off.ctypes.data, dim, _ptr(points), wt, _ptr(weights),
                                  it.ctypes.data, tolerance, MODES[mode], ctypes.c_void_p(s), int(repeats),
                                  ctypes.byref(best))
    _check(rc)
    return best.as_dict()


# ---------------------------------------------------------------------------
# coupe::imbalance (coupe/src/imbalance.rs): part loads and the imbalance
# metrics computed from them.
# ---------------------------------------------------------------------------
def _loads_dtype(wt):
    return {COUPE_INT: np.int32, COUPE_INT64: np.int64, COUPE_DOUBLE: np.float64}[wt]


def _host_ids(partition):
    ids = np.ascontiguousarray(np.asarray(partition))
    if ids.dtype != np.uint64:
        ids = ids.astype(np.uint64)
    return ids


def compute_parts_load(partition, num_parts, weights):
    """Load of each part (compute_parts_load, imbalance.rs:14-39) through
    coupe_gpu_parts_load: an array of num_parts values of the weights' type.
    A part id >= num_parts raises CoupeError (coupe panics)."""
    ids = _host_ids(partition)
    w = _as_weights(weights, len(ids))
    if len(w) != len(ids):
        raise CoupeError(ERR_LEN_MISMATCH)
    wt = _weight_type(w)
    out = np.zeros(num_parts, dtype=_loads_dtype(wt))
    L = lib()
    dw = L.coupe_data_array(len(w), wt, w.ctypes.data)
    try:
        rc = L.coupe_gpu_parts_load(ids.ctypes.data, num_parts, dw, out.ctypes.data)
    finally:
        L.coupe_data_free(dw)
    _check(rc)
    return out


def imbalance(num_parts, partition, weights):
    """coupe::imbalance::imbalance (imbalance.rs:41-77) through
    coupe_gpu_imbalance: max over parts of (load - ideal) / ideal."""
    ids = _host_ids(partition)
    w = _as_weights(weights, len(ids))
    if len(w) != len(ids):
        raise CoupeError(ERR_LEN_MISMATCH)
    out = ctypes.c_double(0.0)
    L = lib()
    dw = L.coupe_data_array(len(w), _weight_type(w), w.ctypes.data)
    try:
        rc = L.coupe_gpu_imbalance(num_parts, ids.ctypes.data, dw, ctypes.byref(out))
    finally:
        L.coupe_data_free(dw)
    _check(rc)
    return out.value


def max_imbalance(num_parts, partition, weights):
    """coupe::imbalance::max_imbalance (imbalance.rs:94-105): largest load
    minus smallest load, in the weights' type (0 without parts)."""
    loads = compute_parts_load(partition, num_parts, weights)
    if len(loads) == 0:
        return loads.dtype.type(0)
    with np.errstate(over="ignore"):
        return loads.max() - loads.min()


def imbalance_target(targets, partition, weights):
    """coupe::imbalance::imbalance_target (imbalance.rs:79-92): the largest
    load - target over the parts (len(targets) parts; 0 without parts)."""
    t = np.asarray(targets)
    loads = compute_parts_load(partition, len(t), weights)
    if len(loads) == 0:
        return loads.dtype.type(0)
    with np.errstate(over="ignore"):
        return (loads - t.astype(loads.dtype)).max()


def _device_weights(weights):
    import torch
    return {torch.int32: COUPE_INT, torch.int64: COUPE_INT64, torch.float64: COUPE_DOUBLE}[weights.dtype]


def parts_load_device(part_ids, weights, num_parts, stream=None):
    """compute_parts_load on CUDA tensors (part_ids int64/uint64 (N,),
    weights int32/int64/float64 (N,)); returns a host numpy array."""
    import torch
    wt = _device_weights(weights)
    out = np.zeros(num_parts, dtype=_loads_dtype(wt))
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    rc = lib().coupe_gpu_parts_load_device(_ptr(part_ids), part_ids.numel(), wt, _ptr(weights), num_parts,
                                           out.ctypes.data, ctypes.c_void_p(s))
    _check(rc)
    return out


def imbalance_device(num_parts, part_ids, weights, stream=None):
    """coupe::imbalance::imbalance on CUDA tensors."""
    import torch
    wt = _device_weights(weights)
    out = ctypes.c_double(0.0)
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    rc = lib().coupe_gpu_imbalance_device(num_parts, _ptr(part_ids), part_ids.numel(), wt, _ptr(weights),
                                          ctypes.byref(out), ctypes.c_void_p(s))
    _check(rc)
    return out.value


class Grid:
    """A 2D or 3D cartesian grid (coupe::Grid, coupe/src/cartesian/mod.rs):
    cell (x, y[, z]) is entry x + size[0] * (y + size[1] * z) of the weights
    and of the partition."""

    def __init__(self, *size):
        if len(size) == 1 and not np.isscalar(size[0]):
            size = tuple(size[0])
        self.size = tuple(int(v) for v in size)

    @classmethod
    def new_2d(cls, width, height):
        return cls(width, height)

    @classmethod
    def new_3d(cls, width, height, depth):
        return cls(width, height, depth)

    def __len__(self):
        return int(np.prod(self.size))

    def rcb(self, partition, weights, iter_count, threads=None):
        """Grid::rcb through coupe_gpu_grid_rcb: writes ids in
        [0, 2**iter_count) into `partition` (uint64, one per cell).  The
        weighted median replays `threads` rayon workers (default: the host's
        CPU count, what a default rayon pool uses; at least 2)."""
        if threads is None:
            threads = max(2, os.cpu_count() or 2)
        w = _as_weights(weights, len(self))
        if partition.dtype != np.uint64 or not partition.flags.c_contiguous:
            raise TypeError("partition must be a contiguous uint64 array")
        if len(partition) != len(w):
            raise CoupeError(ERR_LEN_MISMATCH)
        sz = np.ascontiguousarray(np.asarray(self.size, dtype=np.uint64))
        L = lib()
        dw = L.coupe_data_array(len(w), _weight_type(w), w.ctypes.data)
        try:
            rc = L.coupe_gpu_grid_rcb(partition.ctypes.data, len(self.size), sz.ctypes.data, dw, iter_count,
                                      int(threads))
        finally:
            L.coupe_data_free(dw)
        _check(rc)


def grid_rcb_device(part_ids, weights, size, iter_count, threads, stream=None):
    """Grid::rcb on CUDA tensors: part_ids int64/uint64 and weights
    int32/int64/float64, one per cell of the grid `size`."""
    import torch
    wt = {torch.int32: COUPE_INT, torch.int64: COUPE_INT64, torch.float64: COUPE_DOUBLE}[weights.dtype]
    sz = np.ascontiguousarray(np.asarray(size, dtype=np.uint64))
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    rc = lib().coupe_gpu_grid_rcb_device(_ptr(part_ids), len(sz), sz.ctypes.data, wt, _ptr(weights), iter_count,
                                         int(threads), ctypes.c_void_p(s))
    _check(rc)


def barycentres_device(coords, nodes, stream=None):
    """Element barycentres on CUDA tensors (mesh-part's points,
    tools/lib/lib.rs:511-539): coords float64 (n_nodes, D), nodes int64 or
    uint64 (n_elements, k) 0-based; returns a float64 (n_elements, D) tensor.
    Bit-identical to coupe's sums in node order divided by k."""
    import torch
    n_nodes, dim = coords.shape
    n_el, k = nodes.shape
    out = torch.empty((n_el, dim), dtype=torch.float64, device=coords.device)
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    rc = lib().coupe_gpu_barycentres(dim, n_nodes, _ptr(coords), n_el, k, _ptr(nodes), _ptr(out), ctypes.c_void_p(s))
    _check(rc)
    return out


def barycentres_host(coords, nodes):
    """barycentres_device on host arrays (uploaded, computed on the GPU,
    read back)."""
    import torch
    c = torch.from_numpy(np.ascontiguousarray(coords, dtype=np.float64)).cuda()
    v = torch.from_numpy(np.ascontiguousarray(np.asarray(nodes).astype(np.int64, copy=False))).cuda()
    if v.dim() != 2 or v.shape[0] == 0:
        return np.zeros((0 if v.dim() != 2 else v.shape[0], c.shape[1]))
    return barycentres_device(c, v).cpu().numpy()


def rib_device(part_ids, points, weights, iter_count, tolerance, mode="ref32", stream=None,
               weighted_inertia=False):
    """Rib on CUDA tensors (see rcb_device).  weighted_inertia=True weighs
    the inertia matrix by the weights (an opt-in; coupe's is unweighted)."""
    import torch
    n, dim = points.shape
    wt = {torch.int32: COUPE_INT, torch.int64: COUPE_INT64, torch.float64: COUPE_DOUBLE}[weights.dtype]
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    m = MODES[mode] | (WEIGHTED_INERTIA if weighted_inertia else 0)
    rc = lib().coupe_gpu_rib_device(_ptr(part_ids), n, dim, _ptr(points), wt, _ptr(weights), iter_count,
                                    tolerance, m, ctypes.c_void_p(s))
    _check(rc)


def rib_matrix_device(points, stream=None, weights=None):
    """The Rib basis change (obb_to_aabb) of CUDA float64 points (N, D); with
    `weights` (a CUDA tensor) the weighted inertia's (an opt-in)."""
    import torch
    n, dim = points.shape
    out = np.zeros((dim, dim), dtype=np.float64)
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    if weights is None:
        _check(lib().coupe_gpu_rib_matrix(n, dim, _ptr(points), out.ctypes.data, ctypes.c_void_p(s)))
    else:
        wt = {torch.int32: COUPE_INT, torch.int64: COUPE_INT64, torch.float64: COUPE_DOUBLE}[weights.dtype]
        _check(lib().coupe_gpu_rib_matrix_weighted(n, dim, _ptr(points), wt, _ptr(weights), out.ctypes.data,
                                                   ctypes.c_void_p(s)))
    return out


@dataclass
class MultiJagged:
    """coupe::MultiJagged (coupe/src/algorithms/multi_jagged.rs:368-385):
    part_count parts in at most max_iter iterations.  partition(part_ids,
    (points, weights)) with float64 points (N, D) and float64 weights."""
    part_count: int
    max_iter: int

    def partition(self, part_ids, data):
        points, weights = data
        pts = np.ascontiguousarray(points, dtype=np.float64)
        if pts.ndim != 2:
            raise ValueError("points must be (N, D)")
        w = (np.full(len(pts), weights, dtype=np.float64) if np.isscalar(weights)
             else np.ascontiguousarray(weights, dtype=np.float64))
        if part_ids.dtype not in (np.uint64, np.int64) or not part_ids.flags.c_contiguous:
            raise TypeError("part_ids must be a contiguous uint64/int64 array")
        L = lib()
        dp = L.coupe_data_array(len(pts), COUPE_DOUBLE, pts.ctypes.data)
        dw = L.coupe_data_array(len(w), COUPE_DOUBLE, w.ctypes.data)
        try:
            rc = L.coupe_gpu_multi_jagged(part_ids.ctypes.data, pts.shape[1], dp, dw, self.part_count,
                                          self.max_iter)
        finally:
            L.coupe_data_free(dp)
            L.coupe_data_free(dw)
        _check(rc)


def multi_jagged_device(part_ids, points, weights, part_count, max_iter, stream=None):
    """MultiJagged on CUDA tensors: part_ids int64/uint64 (N,), points
    float64 (N, D), weights float64 (N,)."""
    import torch
    n, dim = points.shape
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    rc = lib().coupe_gpu_multi_jagged_device(_ptr(part_ids), n, dim, _ptr(points), _ptr(weights), part_count,
                                             max_iter, ctypes.c_void_p(s))
    _check(rc)


def axis_sort_device(points, coord, stream=None):
    """coupe's axis_sort of 0..N-1 along `coord` on CUDA float64 points
    (N, D); returns an int64 tensor of point indices (ties in index order)."""
    import torch
    n, dim = points.shape
    out = torch.empty(n, dtype=torch.int64, device=points.device)
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    _check(lib().coupe_gpu_axis_sort_device(_ptr(out), n, dim, _ptr(points), coord, ctypes.c_void_p(s)))
    return out
