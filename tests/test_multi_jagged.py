"""axis_sort and MultiJagged (coupe/src/algorithms/recursive_bisection.rs:
815-827, coupe/src/algorithms/multi_jagged.rs).

CPU: the oracle against the reference's own tests (test_axis_sort_x / _y,
recursive_bisection.rs:1021-1039; the MultiJagged doctest, multi_jagged.rs:
333-365; test_split_at_mut_many, :416-433), properties of the partition
scheme, and the C ABI's argument checks.  GPU: the sort against the golden
orders and the oracle; MultiJagged ids identical to the oracle's for unit and
float weights, 2D and 3D, part counts that need fat parts, empty parts and
the error paths; at a few million points, size-independent properties.
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "reference_known_answers.json")))


def _leaves(scheme):
    if scheme["num_splits"] == 0:
        return 1
    return sum(_leaves(c) for c in scheme["next"])


def _depth(scheme):
    if scheme["num_splits"] == 0:
        return 0
    return 1 + max(_depth(c) for c in scheme["next"])


# ------------------------------------------------------------------ CPU
@pytest.mark.parametrize("case", ["axis_sort_x", "axis_sort_y"])
def test_oracle_axis_sort_golden(case):
    import multi_jagged as mj
    c = GOLDEN[case]
    pts = np.asarray(c["points"])
    assert mj.axis_sort(pts, np.arange(len(pts)), c["coord"]).tolist() == c["expect"]


def test_oracle_split_at_mut_many_golden():
    import multi_jagged as mj
    c = GOLDEN["split_at_mut_many"]
    parts = mj.split_at_mut_many(list(range(c["len"])), c["positions"])
    assert [list(p) for p in parts] == c["expect"]


def test_oracle_doctest_distinct_ids():
    import multi_jagged as mj
    c = GOLDEN["multi_jagged_doctest"]
    ids = mj.multi_jagged(np.asarray(c["points"]), np.full(9, 4.2), c["part_count"], c["max_iter"])
    assert sorted(ids.tolist()) == list(range(9))


@pytest.mark.parametrize("parts", [1, 2, 3, 5, 7, 9, 16, 17, 100, 1000, 4097])
@pytest.mark.parametrize("iters", [1, 2, 3, 4, 7])
def test_oracle_scheme_shape(parts, iters):
    """The scheme has part_count leaves, at most max_iter splitting levels,
    and every node's modifiers add up to 1."""
    import multi_jagged as mj
    s = mj.partition_scheme(parts, iters)
    assert _leaves(s) == parts
    assert _depth(s) <= iters

    def walk(node):
        assert abs(sum(node["modifiers"]) - 1.0) < 1e-12
        assert len(node["modifiers"]) == node["num_splits"] + 1
        for c in node["next"] or []:
            walk(c)
    walk(s)


def test_oracle_scheme_errors():
    import multi_jagged as mj
    with pytest.raises(ValueError):
        mj.partition_scheme(3, 0)
    assert mj.partition_scheme(1, 0)["num_splits"] == 0


def test_oracle_balance_property():
    """Unit weights: every part holds n / part_count points to within one
    point per iteration."""
    import multi_jagged as mj
    rng = np.random.default_rng(3)
    pts = rng.random((3000, 2))
    for parts, iters in [(5, 2), (12, 3), (7, 1)]:
        ids = mj.multi_jagged(pts, np.ones(3000), parts, iters)
        counts = np.bincount(ids, minlength=parts)
        assert len(counts) == parts
        assert np.abs(counts - 3000 / parts).max() <= iters + 1


def test_abi_checks(coupe):
    L = coupe.lib()
    pts = np.zeros((4, 2))
    part = np.zeros(4, dtype=np.uint64)
    wi = np.ones(4, dtype=np.int64)
    wd = np.ones(3)
    dp = L.coupe_data_array(4, coupe.COUPE_DOUBLE, pts.ctypes.data)
    dwi = L.coupe_data_array(4, coupe.COUPE_INT64, wi.ctypes.data)
    dwd = L.coupe_data_array(3, coupe.COUPE_DOUBLE, wd.ctypes.data)
    try:
        assert L.coupe_gpu_multi_jagged(part.ctypes.data, 2, dp, dwd, 2, 1) == coupe.ERR_LEN_MISMATCH
        assert L.coupe_gpu_multi_jagged(part.ctypes.data, 2, dp, dwi, 2, 1) == coupe.ERR_BAD_TYPE
        assert L.coupe_gpu_multi_jagged(part.ctypes.data, 0, dp, dwi, 2, 1) in (coupe.ERR_BAD_DIMENSION,
                                                                                coupe.ERR_BAD_TYPE)
        assert L.coupe_gpu_axis_sort_device(None, 4, 2, None, 2, None) == coupe.ERR_BAD_DIMENSION
        assert L.coupe_gpu_multi_jagged_device(None, 4, 0, None, None, 2, 1, None) == coupe.ERR_BAD_DIMENSION
        assert L.coupe_gpu_multi_jagged_device(None, 0, 2, None, None, 2, 1, None) == coupe.ERR_OK
    finally:
        for d in (dp, dwi, dwd):
            L.coupe_data_free(d)


# ------------------------------------------------------------------ GPU
def _cuda(x, dtype=None):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x if dtype is None else x.astype(dtype))).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["axis_sort_x", "axis_sort_y"])
def test_gpu_axis_sort_golden(coupe, case):
    c = GOLDEN[case]
    out = coupe.axis_sort_device(_cuda(np.asarray(c["points"], dtype=np.float64)), c["coord"])
    assert out.cpu().tolist() == c["expect"]


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_gpu_axis_sort_matches_oracle(coupe, dim):
    import multi_jagged as mj
    rng = np.random.default_rng(dim)
    pts = rng.standard_normal((300_000, dim))
    pts[::7, 0] = np.round(pts[::7, 0], 1)  # ties: both keep index order
    pts[5, 0], pts[6, 0] = -0.0, 0.0
    for coord in range(dim):
        got = coupe.axis_sort_device(_cuda(pts), coord).cpu().numpy()
        want = mj.axis_sort(pts, np.arange(len(pts)), coord)
        np.testing.assert_array_equal(got, want)


@pytest.mark.gpu
def test_gpu_doctest(coupe):
    """The MultiJagged doctest through the host API: nine distinct ids."""
    import multi_jagged as mj
    c = GOLDEN["multi_jagged_doctest"]
    pts = np.asarray(c["points"], dtype=np.float64)
    ids = np.zeros(9, dtype=np.uint64)
    coupe.MultiJagged(part_count=c["part_count"], max_iter=c["max_iter"]).partition(ids, (pts, 4.2))
    assert sorted(ids.tolist()) == list(range(9))
    np.testing.assert_array_equal(ids.astype(np.int64), mj.multi_jagged(pts, np.full(9, 4.2), 9, 4))


CASES = [(2, 1), (3, 1), (5, 2), (7, 3), (9, 4), (16, 2), (33, 3), (64, 6), (100, 2), (257, 3)]


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("weights", ["unit", "float", "int_valued"])
@pytest.mark.parametrize("parts,iters", CASES)
def test_gpu_matches_oracle(coupe, dim, weights, parts, iters):
    import multi_jagged as mj
    rng = np.random.default_rng(parts * 31 + iters * 7 + dim)
    n = 20_000
    pts = rng.random((n, dim))
    w = {"unit": np.ones(n), "float": rng.random(n) * 10 + 0.01,
         "int_valued": rng.integers(1, 100, n).astype(np.float64)}[weights]
    want = mj.multi_jagged(pts, w, parts, iters)
    part = _cuda(np.zeros(n, dtype=np.int64))
    coupe.multi_jagged_device(part, _cuda(pts), _cuda(w), parts, iters)
    np.testing.assert_array_equal(part.cpu().numpy(), want)


@pytest.mark.gpu
def test_gpu_host_api_matches_device(coupe):
    rng = np.random.default_rng(11)
    pts = rng.random((50_000, 3))
    w = rng.random(50_000)
    host = np.zeros(50_000, dtype=np.uint64)
    coupe.MultiJagged(part_count=24, max_iter=3).partition(host, (pts, w))
    dev = _cuda(np.zeros(50_000, dtype=np.int64))
    coupe.multi_jagged_device(dev, _cuda(pts), _cuda(w), 24, 3)
    np.testing.assert_array_equal(host.astype(np.int64), dev.cpu().numpy())


@pytest.mark.gpu
@pytest.mark.parametrize("n,parts,iters", [(1, 1, 1), (1, 4, 2), (5, 9, 2), (10, 64, 3), (3, 3, 1)])
def test_gpu_small_and_empty_parts(coupe, n, parts, iters):
    """Fewer points than parts: some parts stay empty (coupe panics on a
    split of an empty part; here it yields empty children)."""
    import multi_jagged as mj
    rng = np.random.default_rng(n + parts)
    pts = rng.random((n, 2))
    w = np.ones(n)
    want = mj.multi_jagged(pts, w, parts, iters)
    part = _cuda(np.zeros(n, dtype=np.int64))
    coupe.multi_jagged_device(part, _cuda(pts), _cuda(w), parts, iters)
    np.testing.assert_array_equal(part.cpu().numpy(), want)


@pytest.mark.gpu
def test_gpu_errors(coupe):
    pts = _cuda(np.random.default_rng(0).random((100, 2)))
    part = _cuda(np.zeros(100, dtype=np.int64))
    with pytest.raises(coupe.CoupeError) as e:
        coupe.multi_jagged_device(part, pts, _cuda(np.ones(100)), 0, 2)
    assert e.value.code == coupe.ERR_BAD_TYPE
    with pytest.raises(coupe.CoupeError) as e:
        coupe.multi_jagged_device(part, pts, _cuda(np.ones(100)), 3, 0)
    assert e.value.code == coupe.ERR_NOT_FOUND
    w = np.ones(100)
    w[17] = -1.0
    with pytest.raises(coupe.CoupeError) as e:
        coupe.multi_jagged_device(part, pts, _cuda(w), 4, 2)
    assert e.value.code == coupe.ERR_NEG_VALUES
    w[17] = np.inf
    with pytest.raises(coupe.CoupeError) as e:
        coupe.multi_jagged_device(part, pts, _cuda(w), 4, 2)
    assert e.value.code == coupe.ERR_BAD_TYPE
    # the context stays usable after the errors
    coupe.multi_jagged_device(part, pts, _cuda(np.ones(100)), 4, 2)
    assert sorted(set(part.cpu().tolist())) == [0, 1, 2, 3]


@pytest.mark.gpu
@pytest.mark.parametrize("parts,iters", [(1000, 3), (4096, 2)])
def test_gpu_large_properties(coupe, parts, iters):
    """4M points: every id in range and used, unit-weight parts within one
    point per iteration of n / part_count, and the partition does not depend
    on the order of the input points (distinct coordinates)."""
    import torch
    rng = np.random.default_rng(parts)
    n = 4_000_000
    pts = rng.random((n, 3))
    dpts = _cuda(pts)
    part = torch.zeros(n, dtype=torch.int64, device="cuda")
    coupe.multi_jagged_device(part, dpts, torch.ones(n, dtype=torch.float64, device="cuda"), parts, iters)
    counts = torch.bincount(part, minlength=parts).cpu().numpy()
    assert len(counts) == parts
    assert np.abs(counts - n / parts).max() <= iters + 1
    perm = rng.permutation(n)
    part2 = torch.zeros(n, dtype=torch.int64, device="cuda")
    coupe.multi_jagged_device(part2, _cuda(pts[perm]), torch.ones(n, dtype=torch.float64, device="cuda"), parts,
                              iters)
    np.testing.assert_array_equal(part2.cpu().numpy(), part.cpu().numpy()[perm])
