"""Failure handling, tested without faulting, trapping or hanging a GPU.

- A reorder chunk's look-back wait (a bounded spin on its predecessor's
  published prefix) is made to run out by a poll limit of 0: the call must
  fail with COUPE_ERR_CRASH and the look-back error bit, and the next call,
  with the default limit, must give the oracle's ids (the context stays
  usable).
- An allocation failure is injected on the host by a workspace cap: the call
  fails with COUPE_ERR_ALLOC before allocating, and succeeds once the cap is
  lifted (coupe-ffi maps allocation failures to COUPE_ERR_ALLOC,
  coupe-ffi/src/lib.rs:27-33, 318-321).
- coupe_data_fn data sets (coupe-ffi/include/coupe.h:150-188): the callback
  may be called from any thread, in any order, more than once; results equal
  the array data set's.
- Concurrent callers (coupe.h:117-123): several threads calling coupe_rcb at
  once on different inputs each get their own input's ids.
"""
import ctypes
import re
import threading

import numpy as np
import pytest


def _points(n, seed, dim=3):
    rng = np.random.default_rng(seed)
    return rng.random((n, dim)) * 10.0, rng.integers(1, 100, size=n, dtype=np.int64)


def test_options_round_trip(coupe):
    """The failure knobs are options like the scheduling ones; unknown names
    are rejected."""
    for name in ("lookback_spin_limit", "workspace_limit_mb"):
        old = coupe.get_option(name)
        assert old >= 0
        coupe.set_option(name, old)
        assert coupe.get_option(name) == old
    with pytest.raises(coupe.CoupeError):
        coupe.set_option("no_such_option", 1)


@pytest.mark.gpu
def test_lookback_wait_runs_out_then_recovers(coupe, oracle_mod):
    pts, w = _points(2_000_000, 31)
    want, _ = oracle_mod.rcb(pts, w, 8, 0.01)
    ids = np.zeros(len(pts), dtype=np.uint64)
    old = coupe.get_option("lookback_spin_limit")
    coupe.set_option("lookback_spin_limit", 0)
    try:
        with pytest.raises(coupe.CoupeError) as e:
            coupe.Rcb(iter_count=8, tolerance=0.01).partition(ids, (pts, w))
    finally:
        coupe.set_option("lookback_spin_limit", old)
    assert e.value.code == coupe.ERR_CRASH
    m = re.search(r"device check failed \(code (\d+)", str(e.value))
    assert m and int(m.group(1)) & 1, str(e.value)  # ERR_LOOKBACK_TIMEOUT
    ids[:] = 0
    coupe.Rcb(iter_count=8, tolerance=0.01).partition(ids, (pts, w))
    assert (ids == want).all()


@pytest.mark.gpu
def test_workspace_cap_gives_alloc_error_then_recovers(coupe, oracle_mod):
    pts, w = _points(1_000_000, 32)
    want, _ = oracle_mod.rcb(pts, w, 6, 0.01)
    ids = np.zeros(len(pts), dtype=np.uint64)
    old = coupe.get_option("workspace_limit_mb")
    coupe.set_option("workspace_limit_mb", 1)
    try:
        with pytest.raises(coupe.CoupeError) as e:
            coupe.Rcb(iter_count=6, tolerance=0.01).partition(ids, (pts, w))
    finally:
        coupe.set_option("workspace_limit_mb", old)
    assert e.value.code == coupe.ERR_ALLOC
    assert "workspace_limit_mb" in str(e.value)
    coupe.Rcb(iter_count=6, tolerance=0.01).partition(ids, (pts, w))
    assert (ids == want).all()


@pytest.mark.gpu
def test_data_fn_callbacks(coupe, oracle_mod):
    L = coupe.lib()
    pts, w = _points(30_000, 33)
    want, _ = oracle_mod.rcb(pts, w, 7, 0.02)
    calls = {"points": 0, "weights": 0}
    threads = set()
    lock = threading.Lock()
    pbase, wbase = pts.ctypes.data, w.ctypes.data

    def p_ith(ctx, i):
        with lock:
            calls["points"] += 1
            threads.add(threading.get_ident())
        return pbase + i * 3 * 8

    def w_ith(ctx, i):
        with lock:
            calls["weights"] += 1
        return wbase + i * 8

    cp, cw = coupe.I_TH(p_ith), coupe.I_TH(w_ith)
    dp = L.coupe_data_fn(None, len(pts), coupe.COUPE_DOUBLE, cp)
    dw = L.coupe_data_fn(None, len(w), coupe.COUPE_INT64, cw)
    ids = np.zeros(len(pts), dtype=np.uint64)
    try:
        for fn in (L.coupe_rcb, L.coupe_rcb):  # twice: a data set may be read again
            ids[:] = 0
            assert fn(ids.ctypes.data, 3, dp, dw, 7, 0.02) == coupe.ERR_OK
            assert (ids == want).all()
    finally:
        L.coupe_data_free(dp)
        L.coupe_data_free(dw)
    assert calls["points"] >= 2 * len(pts) and calls["weights"] >= 2 * len(w)
    # constant weights through the same call
    dp = L.coupe_data_fn(None, len(pts), coupe.COUPE_DOUBLE, cp)
    one = np.array([1], dtype=np.int64)
    dc = L.coupe_data_constant(len(pts), coupe.COUPE_INT64, one.ctypes.data)
    try:
        assert L.coupe_rcb(ids.ctypes.data, 3, dp, dc, 5, 0.05) == coupe.ERR_OK
    finally:
        L.coupe_data_free(dp)
        L.coupe_data_free(dc)
    want1, _ = oracle_mod.rcb(pts, np.ones(len(pts), dtype=np.int64), 5, 0.05)
    assert (ids == want1).all()


@pytest.mark.gpu
def test_concurrent_callers(coupe, oracle_mod):
    L = coupe.lib()
    inputs = [_points(150_000 + 1000 * k, 40 + k, dim=2 + (k % 2)) for k in range(4)]
    wants = [oracle_mod.rcb(p, w, 7 + k % 3, 0.01)[0] for k, (p, w) in enumerate(inputs)]
    errors = []

    def worker(k):
        p, w = inputs[k]
        for rep in range(3):
            ids = np.zeros(len(p), dtype=np.uint64)
            dp = L.coupe_data_array(len(p), coupe.COUPE_DOUBLE, p.ctypes.data)
            dw = L.coupe_data_array(len(w), coupe.COUPE_INT64, w.ctypes.data)
            rc = L.coupe_rcb(ids.ctypes.data, p.shape[1], dp, dw, 7 + k % 3, 0.01)
            L.coupe_data_free(dp)
            L.coupe_data_free(dw)
            if rc != coupe.ERR_OK or not (ids == wants[k]).all():
                errors.append((k, rep, rc, int((ids != wants[k]).sum())))

    ts = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
