"""GPU parity: libcoupe_gpu.so (through its C ABI) against the oracle.

Integer weights: part ids must be bit-identical.  f64 weights: identical to
the oracle run with the same 128-bit fixed-point sums (the GPU's summation),
and compared with the oracle's sequential f64 sums by id agreement.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gpu(coupe, pts, w, iters, tol, mode="ref32", rib=False):
    ids = np.zeros(len(pts), dtype=np.uint64)
    (coupe.Rib if rib else coupe.Rcb)(iter_count=iters, tolerance=tol, mode=mode).partition(ids, (pts, w))
    return ids


def _oracle_mode(mode):
    return 1 if mode == "f64" else 0


# ---------------------------------------------------------------------------
# Known answers of the reference's own tests, through coupe_rcb / coupe_rib.
# ---------------------------------------------------------------------------
def test_ffi_example_rcb_c(coupe):
    """coupe-ffi/examples/rcb.c: 4 points, constant int weight 1."""
    L = coupe.lib()
    pts = np.array([[0.0, 0.0], [0.0, 1.0], [1.0, 0.0], [1.0, 1.0]])
    one = ctypes.c_int(1)
    dp = L.coupe_data_array(4, coupe.COUPE_DOUBLE, pts.ctypes.data)
    dw = L.coupe_data_constant(4, coupe.COUPE_INT, ctypes.addressof(one))
    part = np.zeros(4, dtype=np.uint64)
    assert L.coupe_rcb(part.ctypes.data, 2, dp, dw, 1, 0.05) == 0
    assert part.tolist() == [0, 0, 1, 1]
    assert L.coupe_rcb(part.ctypes.data, 2, dp, dw, 2, 0.05) == 0
    assert part.tolist() == [0, 1, 2, 3]
    L.coupe_data_free(dp)
    L.coupe_data_free(dw)


def test_rcb_basic(coupe):
    """recursive_bisection.rs:1077-1115 (test_rcb_basic)."""
    pts = np.array([[-1.3, 6.0], [2.0, -4.0], [1.0, 1.0], [-3.0, -2.5],
                    [-1.3, -0.3], [2.0, 1.0], [-3.0, 1.0], [1.3, -2.0]])
    p = _gpu(coupe, pts, np.ones(8), 2, 0.05)
    assert p[0] == p[6] and p[1] == p[7] and p[2] == p[5] and p[3] == p[4]
    assert sorted(np.bincount(p.astype(np.int64)).tolist()) == [2, 2, 2, 2]


def test_rcb_doctest(coupe):
    """recursive_bisection.rs:739-768: 4 points, 2 iterations, all distinct."""
    pts = np.array([[1.0, 1.0], [-1.0, 1.0], [1.0, -1.0], [-1.0, -1.0]])
    p = _gpu(coupe, pts, np.ones(4, np.int32), 2, 0.0)
    assert len(set(p.tolist())) == 4


def test_rib_doctest(coupe):
    """recursive_bisection.rs:862-894: Rib splits along the inertia axis (y)."""
    pts = np.array([[1.0, 10.0], [-1.0, 10.0], [1.0, -10.0], [-1.0, -10.0]])
    p = _gpu(coupe, pts, np.ones(4, np.int32), 1, 0.0, rib=True)
    assert p[0] == p[1] and p[2] == p[3] and p[1] != p[2]


# ---------------------------------------------------------------------------
# Random parity against the oracle
# ---------------------------------------------------------------------------
CASES = [
    # n, dim, weight kind, iters, tol, seed
    (1, 2, "i64", 3, 0.05, 1),
    (2, 3, "i64", 2, 0.05, 2),
    (7, 2, "i32", 3, 0.0, 3),
    (100, 2, "i64", 5, 0.05, 4),
    (1000, 3, "i32", 6, 0.01, 5),
    (4097, 2, "f64", 4, 0.02, 6),
    (20000, 3, "i64", 8, 0.01, 7),
    (100000, 2, "i64", 10, 0.001, 8),
    (100000, 3, "f64", 7, 0.005, 9),
    (250000, 3, "i64", 9, 0.01, 10),
    (3000, 2, "i64", 14, 0.05, 11),   # deep: singletons at the bottom
    (50000, 3, "i32", 12, -1.0, 12),  # negative tolerance never stops early
]


def _make(n, dim, wk, seed):
    rng = np.random.default_rng(seed)
    pts = rng.random((n, dim)) * rng.uniform(0.5, 100.0)
    if n > 10:
        pts[: n // 10] = np.round(pts[: n // 10], 1)  # duplicates and ties
    if wk == "i64":
        w = rng.integers(1, 100, size=n, dtype=np.int64)
    elif wk == "i32":
        w = rng.integers(1, 100, size=n, dtype=np.int32)
    else:
        w = rng.lognormal(0.0, 1.0, size=n)
    return pts, w


@pytest.mark.parametrize("mode", ["ref32", "f64"])
@pytest.mark.parametrize("n,dim,wk,iters,tol,seed", CASES)
def test_parity_random(coupe, oracle_mod, n, dim, wk, iters, tol, seed, mode):
    pts, w = _make(n, dim, wk, seed)
    want, st = oracle_mod.rcb(pts, w, iters, tol, mode=_oracle_mode(mode), fsum=oracle_mod.FSUM_FIXED)
    got = _gpu(coupe, pts, w, iters, tol, mode=mode)
    assert st["pivot_ties"] == 0
    mism = int((want != got).sum())
    assert mism == 0, "%d / %d ids differ" % (mism, n)


def test_config1_uniform2d(coupe, oracle_mod):
    """1,000,000 2D points, unit i64 weights, iter_count 3, tol 0.05, seed 0."""
    from coupe_gb300 import workloads
    pts, w, cfg = workloads.uniform2d_unit()
    want, _ = oracle_mod.rcb(pts, w, cfg["iter_count"], cfg["tolerance"], threads=0)
    got = _gpu(coupe, pts, w, cfg["iter_count"], cfg["tolerance"])
    assert (want == got).all()
