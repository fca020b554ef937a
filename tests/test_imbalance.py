"""Part loads and imbalance (coupe::imbalance, coupe/src/imbalance.rs:14-105).

CPU: the oracle's restatement on hand-checked cases and the argument checks of
the C ABI that return before any device work.  GPU: the library's loads and
imbalance against the oracle (bit-identical: integer loads wrap like coupe's
release build, f64 loads are fixed-point sums on both sides), against exact
sums, through the host and the device entry points, on the privatised and the
global-memory paths, and on runs of equal part ids (the warp-sum path).
"""
import ctypes
import math

import numpy as np
import pytest

from coupe_gb300 import workloads


# ---------------------------------------------------------------- CPU: oracle
def test_oracle_known_answers(oracle_mod):
    o = oracle_mod
    # loads 3 and 7 of a total 10 over 2 parts: ideal 5, max (7 - 5) / 5
    assert list(o.parts_load([0, 0, 1, 1], 2, np.array([1, 2, 3, 4]))) == [3, 7]
    assert o.imbalance(2, [0, 0, 1, 1], np.array([1, 2, 3, 4])) == 0.4
    assert o.imbalance(2, [0, 0, 1, 1], np.array([1.0, 2.0, 3.0, 4.0])) == 0.4
    # an empty part has load 0: (0 - 5/3) / (5/3) = -1 is not the maximum
    assert o.imbalance(3, [0, 1, 1], np.array([1, 2, 2])) == (4 - 5 / 3) / (5 / 3)
    # no parts: 0 before any load is computed (imbalance.rs:52-55), even with ids
    assert o.imbalance(0, [0, 0], np.array([1, 1])) == 0.0
    # zero ideal load (no points, or weights summing to 0): 0 (imbalance.rs:60-63)
    assert o.imbalance(3, [], np.array([], dtype=np.int64)) == 0.0
    assert o.imbalance(2, [0, 1], np.array([5, -5])) == 0.0
    # negative total: the formula as written (ideal < 0)
    assert o.imbalance(2, [0, 1], np.array([-1, -3])) == max((-1 - -2) / -2, (-3 - -2) / -2)


def test_oracle_integer_loads_wrap(oracle_mod):
    """c_int loads wrap at 32 bits, int64 loads at 64 (release-build `+=`)."""
    o = oracle_mod
    w32 = np.array([2**31 - 1, 5, -3, 2**31 - 1], dtype=np.int32)
    assert list(o.parts_load([0, 0, 1, 0], 2, w32)) == [3, -3]
    w64 = np.array([2**63 - 1, 2, 7], dtype=np.int64)
    assert list(o.parts_load([0, 0, 1], 2, w64)) == [-(2**63) + 1, 7]


def test_oracle_f64_loads_are_near_exact_sums(oracle_mod):
    rng = np.random.default_rng(3)
    w = rng.lognormal(0.0, 2.0, 20_000)
    ids = rng.integers(0, 37, len(w)).astype(np.uint64)
    loads = oracle_mod.parts_load(ids, 37, w)
    for p in range(37):
        exact = math.fsum(w[ids == p])
        assert abs(loads[p] - exact) <= 1e-12 * abs(exact)


def test_oracle_rejects_out_of_range_ids(oracle_mod):
    with pytest.raises(IndexError):
        oracle_mod.parts_load([0, 3], 3, np.array([1, 1]))


# ---------------------------------------------------- CPU: C ABI before device
def test_abi_checks_without_device_work(coupe):
    L = coupe.lib()
    w = np.ones(4, dtype=np.int64)
    ids = np.zeros(4, dtype=np.uint64)
    dw = L.coupe_data_array(4, coupe.COUPE_INT64, w.ctypes.data)
    out = ctypes.c_double(7.0)
    try:
        # no parts: 0 at once (imbalance.rs:52-55)
        assert L.coupe_gpu_imbalance(0, ids.ctypes.data, dw, ctypes.byref(out)) == coupe.ERR_OK
        assert out.value == 0.0
        assert L.coupe_gpu_imbalance_device(0, None, 4, coupe.COUPE_INT64, None, ctypes.byref(out), None) == 0
        # unknown weight type, NULL results and data sets
        assert L.coupe_gpu_parts_load_device(None, 0, 9, None, 1, None, None) == coupe.ERR_BAD_TYPE
        assert L.coupe_gpu_imbalance(2, ids.ctypes.data, None, ctypes.byref(out)) == coupe.ERR_CRASH
        assert L.coupe_gpu_imbalance(2, ids.ctypes.data, dw, None) == coupe.ERR_CRASH
        assert L.coupe_gpu_parts_load(ids.ctypes.data, 2, dw, None) == coupe.ERR_CRASH
    finally:
        L.coupe_data_free(dw)


# ------------------------------------------------------------------ GPU tests
def _cases(rng):
    n = 200_000
    for P in (1, 7, 1024, 5000, 20_000):
        ids = rng.integers(0, P, n).astype(np.uint64)
        yield P, ids, rng.integers(-50, 1000, n).astype(np.int32)
        yield P, ids, rng.integers(-(2**40), 2**40, n).astype(np.int64)
        yield P, ids, rng.lognormal(0.0, 2.0, n) * rng.choice([-1.0, 1.0], n)


@pytest.mark.gpu
def test_loads_and_imbalance_match_oracle(coupe, oracle_mod):
    """Host entry points: parts privatised in shared memory (up to 12K int /
    3K f64 parts) and in global memory beyond."""
    rng = np.random.default_rng(1)
    for P, ids, w in _cases(rng):
        want = oracle_mod.parts_load(ids, P, w)
        got = coupe.compute_parts_load(ids, P, w)
        assert got.dtype == w.dtype
        assert np.array_equal(got, want), (P, w.dtype)
        assert coupe.imbalance(P, ids, w) == oracle_mod.imbalance(P, ids, w), (P, w.dtype)


@pytest.mark.gpu
def test_device_entry_points_and_runs(coupe, oracle_mod):
    """Device tensors; sorted ids (runs of one part per warp) and a mesh-like
    order take the warp-sum path."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2)
    n, P = 300_001, 300
    for ids in (np.sort(rng.integers(0, P, n)).astype(np.uint64),
                (np.arange(n) // 1000 % P).astype(np.uint64),
                rng.integers(0, P, n).astype(np.uint64)):
        for w in (rng.integers(1, 100, n).astype(np.int64), rng.random(n) + 0.5):
            dids = torch.from_numpy(ids.astype(np.int64)).cuda()
            dw = torch.from_numpy(w).cuda()
            want = oracle_mod.parts_load(ids, P, w)
            assert np.array_equal(coupe.parts_load_device(dids, dw, P), want)
            assert coupe.imbalance_device(P, dids, dw) == oracle_mod.imbalance(P, ids, w)


@pytest.mark.gpu
def test_f64_loads_are_near_exact_sums(coupe):
    rng = np.random.default_rng(4)
    n, P = 400_000, 64
    w = rng.lognormal(0.0, 3.0, n)
    ids = rng.integers(0, P, n).astype(np.uint64)
    got = coupe.compute_parts_load(ids, P, w)
    for p in range(P):
        exact = math.fsum(w[ids == p])
        assert abs(got[p] - exact) <= 1e-12 * abs(exact)
    # the loads sum to the total weight
    assert abs(math.fsum(got) - math.fsum(w)) <= 1e-12 * math.fsum(w)


@pytest.mark.gpu
def test_edge_cases(coupe, oracle_mod):
    L = coupe.lib()
    # no points: zero loads and imbalance 0
    e = np.zeros(0, dtype=np.int64)
    assert np.array_equal(coupe.compute_parts_load(e.astype(np.uint64), 5, e), np.zeros(5, dtype=np.int64))
    assert coupe.imbalance(5, e.astype(np.uint64), e) == 0.0
    # an id out of range; no parts with points; a non-finite weight
    with pytest.raises(coupe.CoupeError):
        coupe.compute_parts_load(np.array([0, 5], dtype=np.uint64), 5, np.array([1, 1]))
    with pytest.raises(coupe.CoupeError):
        coupe.compute_parts_load(np.array([0], dtype=np.uint64), 0, np.array([1]))
    with pytest.raises(coupe.CoupeError):
        coupe.imbalance(2, np.array([0, 1], dtype=np.uint64), np.array([1.0, np.inf]))
    # the context is still usable after those errors
    assert coupe.imbalance(2, np.array([0, 1, 1], dtype=np.uint64), np.array([1, 1, 1])) == (2 - 1.5) / 1.5
    # wrap-around: c_int and int64 loads like coupe's release build
    w32 = np.array([2**31 - 1, 5, -3, 2**31 - 1], dtype=np.int32)
    ids = np.array([0, 0, 1, 0], dtype=np.uint64)
    assert np.array_equal(coupe.compute_parts_load(ids, 2, w32), oracle_mod.parts_load(ids, 2, w32))
    # a constant weight data set (coupe_data_constant)
    n = 10_000
    ids = (np.arange(n) % 3).astype(np.uint64)
    v = np.array([4], dtype=np.int64)
    dw = L.coupe_data_constant(n, coupe.COUPE_INT64, v.ctypes.data)
    out = np.zeros(3, dtype=np.int64)
    try:
        assert L.coupe_gpu_parts_load(ids.ctypes.data, 3, dw, out.ctypes.data) == coupe.ERR_OK
    finally:
        L.coupe_data_free(dw)
    assert list(out) == [4 * 3334, 4 * 3333, 4 * 3333]
    # max_imbalance and imbalance_target from the loads (imbalance.rs:79-105)
    w = np.array([1, 2, 3, 4, 10], dtype=np.int64)
    ids = np.array([0, 0, 1, 1, 2], dtype=np.uint64)
    assert coupe.max_imbalance(3, ids, w) == 10 - 3
    assert coupe.imbalance_target(np.array([2, 2, 2]), ids, w) == 8


@pytest.mark.gpu
def test_imbalance_of_an_rcb_partition(coupe, oracle_mod):
    """After a partition, as coupe's tools check it: the GPU's imbalance of
    the GPU ids equals the oracle's of the same ids and of the oracle's own
    partition (coupe's split rules stop some splits early on clustered
    data: 0.376 here, although each split aims at 1 %)."""
    torch = pytest.importorskip("torch")
    pts, w, cfg = workloads.gaussian_mixture3d(n=1_000_000, seed=5)
    dp = torch.from_numpy(pts).cuda()
    dw = torch.from_numpy(w).cuda()
    ids = torch.zeros(len(pts), dtype=torch.int64, device="cuda")
    coupe.rcb_device(ids, dp, dw, 6, 0.01, mode="f32key_f64band")
    P = int(ids.max().item()) + 1
    got = coupe.imbalance_device(P, ids, dw)
    h_ids = ids.cpu().numpy().astype(np.uint64)
    assert got == oracle_mod.imbalance(P, h_ids, w)
    assert got == coupe.imbalance(P, h_ids, w)
    ref_ids, _ = oracle_mod.rcb(pts, w, 6, 0.01, mode=oracle_mod.F64, threads=0)
    assert got == oracle_mod.imbalance(P, ref_ids, w)
