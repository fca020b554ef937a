"""coupe_gpu_split_noalloc, the allocation-free split of one part, against
the library's Rcb entry point and a numpy stable partition.

This file sorts last so that its GPU tests also run after every other test
of the session (the split's static scratch then follows other calls on the
same device); it passes alone in a fresh process too.
"""
import ctypes
import gc

import numpy as np
import pytest

ERR_OK, ERR_ALLOC = 0, 1


def _split(coupe):
    f = coupe.lib().coupe_gpu_split_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_uint64), ctypes.c_void_p]
    return f


def test_split_rejects_more_than_2_32_points(coupe):
    """Rejected before any memory is touched (the pointers are never used)."""
    f = _split(coupe)
    nl = ctypes.c_uint64(7)
    rc = f(1 << 32, 3, 8, coupe.COUPE_INT64, 8, 0, 0.0, 16, 16, ctypes.byref(nl), None)
    assert rc == ERR_ALLOC
    assert b"2^32 - 1" in coupe.lib().coupe_gpu_last_error()
    assert nl.value == 7


def test_split_empty_and_bad_arguments(coupe):
    f = _split(coupe)
    nl = ctypes.c_uint64(7)
    assert f(0, 2, None, coupe.COUPE_INT, None, 0, 1.0, None, None, ctypes.byref(nl), None) == ERR_OK
    assert nl.value == 0
    assert f(10, 3, 8, coupe.COUPE_INT, 8, 3, 1.0, 16, 16, ctypes.byref(nl), None) != ERR_OK  # coord >= dim
    assert f(10, 4, 8, coupe.COUPE_INT, 8, 0, 1.0, 16, 16, ctypes.byref(nl), None) != ERR_OK  # dimension


def _run(f, torch, dp, dw, wt, coord, cut):
    op = torch.full_like(dp, float("nan"))
    ow = torch.zeros_like(dw)
    nl = ctypes.c_uint64(0)
    rc = f(dp.shape[0], dp.shape[1], dp.data_ptr(), wt, dw.data_ptr(), coord, cut, op.data_ptr(), ow.data_ptr(),
           ctypes.byref(nl), torch.cuda.current_stream().cuda_stream)
    return rc, nl.value, op.cpu().numpy(), ow.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("dim,wk", [(3, "i64"), (2, "f64"), (3, "i32"), (2, "i64")])
def test_split_equals_rcb_first_cut_twice(coupe, dim, wk):
    """The first Rcb cut, found by the existing entry point (coupe_gpu_rcb with
    iter_count 1): splitting at the smallest right coordinate gives exactly
    its left and right sets, stably.  Two calls in a row give the same."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(40 + dim)
    n = 1_000_003
    pts = rng.normal(size=(n, dim)) * 10.0
    pts[rng.integers(0, n, 1000), 0] = 0.5  # ties near the middle
    w = {"i64": lambda: rng.integers(1, 100, n).astype(np.int64),
         "i32": lambda: rng.integers(1, 100, n).astype(np.int32),
         "f64": lambda: rng.lognormal(0.0, 1.0, n)}[wk]()
    ids = np.zeros(n, dtype=np.uint64)
    coupe.Rcb(iter_count=1, tolerance=0.05, mode="f64").partition(ids, (pts, w))
    left = ids == 0
    cut = float(pts[~left, 0].min())
    assert (pts[left, 0] < cut).all()
    want_p = np.concatenate([pts[left], pts[~left]])
    want_w = np.concatenate([w[left], w[~left]])
    wt = {"i64": coupe.COUPE_INT64, "i32": coupe.COUPE_INT, "f64": coupe.COUPE_DOUBLE}[wk]
    f = _split(coupe)
    dp = torch.from_numpy(pts).cuda()
    dw = torch.from_numpy(w).cuda()
    for _ in range(2):
        rc, nl, op, ow = _run(f, torch, dp, dw, wt, 0, cut)
        assert rc == ERR_OK, coupe.lib().coupe_gpu_last_error()
        assert nl == int(left.sum())
        assert np.array_equal(op, want_p)
        assert np.array_equal(ow, want_w)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 2047, 2048, 2049, 300_001, 9_000_000])
def test_split_ragged_sizes_nan_and_signed_zero(coupe, n):
    """Against a numpy stable partition: NaN coordinates go right, -0 == +0,
    ragged tile and chunk ends, a cut on the last axis."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n)
    pts = rng.normal(size=(n, 3))
    k = max(1, n // 50)
    pts[rng.integers(0, n, k), 2] = np.nan
    pts[rng.integers(0, n, k), 2] = -0.0
    pts[rng.integers(0, n, k), 2] = 0.0
    w = rng.integers(-5, 1000, n).astype(np.int64)
    f = _split(coupe)
    dp = torch.from_numpy(pts).cuda()
    dw = torch.from_numpy(w).cuda()
    for cut in (0.0, 0.7, float("nan"), float("inf")):
        mask = pts[:, 2] < cut
        rc, nl, op, ow = _run(f, torch, dp, dw, coupe.COUPE_INT64, 2, cut)
        assert rc == ERR_OK, coupe.lib().coupe_gpu_last_error()
        assert nl == int(mask.sum())
        want_p = np.concatenate([pts[mask], pts[~mask]])
        assert np.array_equal(op, want_p, equal_nan=True)
        assert np.array_equal(np.signbit(op), np.signbit(want_p))
        assert np.array_equal(ow, np.concatenate([w[mask], w[~mask]]))


@pytest.mark.gpu
def test_split_allocates_nothing(coupe):
    """After the first call's set-up, a call changes neither the device's free
    memory (cudaMemGetInfo) nor torch's allocator: the outputs are the
    caller's and the scratch is the library's static array."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    n = 2_000_000
    dp = torch.from_numpy(rng.random((n, 3))).cuda()
    dw = torch.from_numpy(rng.integers(1, 9, n).astype(np.int64)).cuda()
    op = torch.empty_like(dp)
    ow = torch.empty_like(dw)
    f = _split(coupe)
    nl = ctypes.c_uint64(0)
    s = torch.cuda.current_stream().cuda_stream

    def call():
        return f(n, 3, dp.data_ptr(), coupe.COUPE_INT64, dw.data_ptr(), 1, 0.5, op.data_ptr(), ow.data_ptr(),
                 ctypes.byref(nl), s)
    assert call() == ERR_OK  # set-up on this device (if not done already)
    torch.cuda.synchronize()
    # tensors of earlier tests that only a garbage collection frees would
    # change torch's counters in the middle of the measurement
    gc.collect()
    gc.disable()
    try:
        free0, _ = torch.cuda.mem_get_info()
        alloc0, reserved0 = torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
        for _ in range(3):
            assert call() == ERR_OK
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        alloc1, reserved1 = torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
    finally:
        gc.enable()
    assert free1 == free0
    assert alloc1 == alloc0 and reserved1 == reserved0
    assert nl.value == int((dp[:, 1] < 0.5).sum().item())
