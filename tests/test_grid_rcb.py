"""Rcb on a cartesian grid (coupe::Grid::rcb, coupe/src/cartesian/rcb.rs).

CPU: the oracle against the reference's own tests (test_3d, rcb.rs:323-361;
the weighted-median property, rcb.rs:305-321) and the C ABI's argument
checks.  GPU: ids identical to the oracle's for integer and f64 weights,
2D and 3D, several rayon worker counts, uneven sizes and deep trees.
"""
import zlib

import numpy as np
import pytest


# ------------------------------------------------------------------ CPU
@pytest.mark.parametrize("threads", [2, 3, 8, 64])
def test_oracle_reference_test_3d(oracle_mod, threads):
    """rcb.rs:323-361: a 4x4x4 grid of unit weights in 8 parts gives eight
    2x2x2 blocks."""
    ids = oracle_mod.grid_rcb([4, 4, 4], np.ones(64), 3, threads).reshape(4, 4, 4)  # [z, y, x]
    for z in (0, 2):
        for y in (0, 2):
            for x in (0, 2):
                assert len(set(ids[z:z + 2, y:y + 2, x:x + 2].reshape(-1).tolist())) == 1
    assert len(set(ids.reshape(-1).tolist())) == 8


def test_oracle_weighted_median_property(oracle_mod):
    """rcb.rs:305-321: the left weight is the sum of the weights before the
    split position (u32 weights, 2 to 199 of them)."""
    rng = np.random.default_rng(0)
    for _ in range(300):
        n = int(rng.integers(2, 200))
        w = rng.integers(0, 1_000_000, n).astype(np.int64)
        threads = int(rng.integers(2, 33))
        pos, left = oracle_mod.grid_weighted_median(w, int(w.sum()), threads, np.int64)
        assert left == int(w[:pos].sum())


def test_oracle_2d_halves(oracle_mod):
    """Uniform 2D grid, one split: on axis 1 (y), at the middle row."""
    ids = oracle_mod.grid_rcb([6, 8], np.ones(48, dtype=np.int64), 1, 4).reshape(8, 6)
    assert (ids[:4] == 0).all() and (ids[4:] == 1).all()


def test_abi_checks(coupe):
    L = coupe.lib()
    w = np.ones(12, dtype=np.int64)
    part = np.zeros(12, dtype=np.uint64)
    dw = L.coupe_data_array(12, coupe.COUPE_INT64, w.ctypes.data)
    try:
        for size, dim, threads, want in [([3, 4], 2, 4, coupe.ERR_OK), ([3, 4], 1, 4, coupe.ERR_BAD_DIMENSION),
                                         ([3, 4, 1, 1], 4, 4, coupe.ERR_BAD_DIMENSION),
                                         ([0, 4], 2, 4, coupe.ERR_BAD_DIMENSION),
                                         ([3, 5], 2, 4, coupe.ERR_LEN_MISMATCH),
                                         ([3, 4], 2, 1, coupe.ERR_BAD_TYPE)]:
            if want == coupe.ERR_OK:
                continue  # needs a device
            sz = np.asarray(size, dtype=np.uint64)
            assert L.coupe_gpu_grid_rcb(part.ctypes.data, dim, sz.ctypes.data, dw, 2, threads) == want, size
    finally:
        L.coupe_data_free(dw)


# ------------------------------------------------------------------ GPU
CASES = [
    ((64, 48), "i64", 6, 4),
    ((37, 91), "f64", 7, 16),
    ((33, 17, 29), "i32", 8, 2),
    ((40, 40, 40), "f64", 9, 8),
    ((5, 300, 7), "i64", 10, 3),
    ((16, 16, 16), "i64", 12, 6),   # deeper than the grid: empty halves
    ((1, 1), "f64", 3, 4),
]


def _weights(rng, n, kind):
    if kind == "i64":
        return rng.integers(0, 1000, n).astype(np.int64)
    if kind == "i32":
        return rng.integers(-5, 2**20, n).astype(np.int32)
    return rng.lognormal(0.0, 1.5, n)


@pytest.mark.gpu
@pytest.mark.parametrize("size,kind,iters,threads", CASES)
def test_grid_rcb_matches_oracle(coupe, oracle_mod, size, kind, iters, threads):
    rng = np.random.default_rng(zlib.crc32(repr((size, kind)).encode()))
    n = int(np.prod(size))
    w = _weights(rng, n, kind)
    want = oracle_mod.grid_rcb(list(size), w, iters, threads)
    part = np.zeros(n, dtype=np.uint64)
    coupe.Grid(size).rcb(part, w, iters, threads=threads)
    assert np.array_equal(part, want)
    assert int(part.max()) < 2**iters


@pytest.mark.gpu
def test_grid_rcb_device_and_unit_weights(coupe, oracle_mod):
    torch = pytest.importorskip("torch")
    size = (128, 96, 64)
    n = int(np.prod(size))
    w = np.ones(n, dtype=np.int64)
    ids = torch.zeros(n, dtype=torch.int64, device="cuda")
    coupe.grid_rcb_device(ids, torch.from_numpy(w).cuda(), size, 6, 8)
    got = ids.cpu().numpy().astype(np.uint64)
    assert np.array_equal(got, oracle_mod.grid_rcb(list(size), w, 6, 8))
    # unit weights on a grid of even sides: 64 equal boxes
    assert np.bincount(got.astype(np.int64), minlength=64).tolist() == [n // 64] * 64


@pytest.mark.gpu
def test_grid_rcb_errors(coupe):
    with pytest.raises(coupe.CoupeError):
        coupe.Grid(4, 4).rcb(np.zeros(16, dtype=np.uint64), np.r_[np.ones(15), np.inf], 2, threads=4)
    part = np.zeros(16, dtype=np.uint64)
    coupe.Grid(4, 4).rcb(part, np.ones(16), 0, threads=4)  # no split: one part
    assert (part == 0).all()
