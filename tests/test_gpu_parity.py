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
    # the band form decides exactly like the F64 form
    return 1 if mode in ("f64", "f32key_f64band") else 0


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


@pytest.mark.parametrize("mode", ["ref32", "f64", "f32key_f64band"])
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


# ---------------------------------------------------------------------------
# Harder inputs: clusters, planes of equal keys, special values, weights that
# take the general (non-packed) accumulation, integer wrap-around.
# ---------------------------------------------------------------------------
def _check(coupe, oracle_mod, pts, w, iters, tol, mode="ref32", fsum=None, nan_right=False):
    om = _oracle_mode(mode) | (oracle_mod.NAN_RIGHT if nan_right else 0)
    want, st = oracle_mod.rcb(pts, w, iters, tol, mode=om,
                              fsum=oracle_mod.FSUM_FIXED if fsum is None else fsum)
    got = _gpu(coupe, pts, w, iters, tol, mode=mode)
    assert st["pivot_ties"] == 0
    mism = int((want != got).sum())
    assert mism == 0, "%d / %d ids differ" % (mism, len(pts))
    return got, st


@pytest.mark.parametrize("mode", ["ref32", "f64", "f32key_f64band"])
def test_gaussian_clusters(coupe, oracle_mod, mode):
    from coupe_gb300 import workloads
    pts, w, cfg = workloads.gaussian_mixture3d(n=400_000, seed=3)
    _check(coupe, oracle_mod, pts, w, cfg["iter_count"], cfg["tolerance"], mode)


@pytest.mark.parametrize("mode", ["ref32", "f64", "f32key_f64band"])
def test_planes_f64_weights(coupe, oracle_mod, mode):
    from coupe_gb300 import workloads
    pts, w, cfg = workloads.planes3d_lognormal(n=300_000, seed=4)
    _check(coupe, oracle_mod, pts, w, 9, cfg["tolerance"], mode)


def test_all_points_identical(coupe, oracle_mod):
    pts = np.full((5000, 3), 1.25)
    w = np.ones(5000, dtype=np.int64)
    _check(coupe, oracle_mod, pts, w, 6, 0.05)


def test_special_values(coupe, oracle_mod):
    rng = np.random.default_rng(21)
    pts = rng.standard_normal((20000, 2))
    pts[::97, 0] = np.inf
    pts[5::101, 1] = -np.inf
    pts[7::89, 0] = np.nan
    pts[::53, 1] = -0.0
    pts[3::59, 0] = 1e300   # beyond f32: key becomes inf in REF32
    pts[11::61, 1] = 1e-310  # subnormal f64
    w = rng.integers(1, 5, size=len(pts), dtype=np.int64)
    for mode in ("ref32", "f64", "f32key_f64band"):
        _check(coupe, oracle_mod, pts, w, 7, 0.02, mode)
    # finite bounding box: signed zeros and subnormals
    pts = rng.standard_normal((20000, 2))
    pts[::53, 1] = -0.0
    pts[::57, 1] = 0.0
    pts[11::61, 1] = 1e-310
    pts[13::67, 0] = -1e-40  # a subnormal f32 key
    for mode in ("ref32", "f64", "f32key_f64band"):
        got, _ = _check(coupe, oracle_mod, pts, w, 7, 0.02, mode)
        assert len(set(got.tolist())) > 64


def test_nan_coordinates(coupe, oracle_mod):
    """NaN keys: coupe's Hoare partition puts a NaN-keyed item left or right
    depending on where it sits in the segment; the GPU sends it right.  Exact
    against the oracle with that rule, and close to coupe's own placement."""
    rng = np.random.default_rng(26)
    pts = rng.standard_normal((20000, 2))
    pts[7::89, 0] = np.nan
    pts[3::97, 1] = np.nan
    w = rng.integers(1, 5, size=len(pts), dtype=np.int64)
    for mode in ("f32key_f64band", "f64", "ref32"):
        got, _ = _check(coupe, oracle_mod, pts, w, 7, 0.02, mode, nan_right=True)
    ref, _ = oracle_mod.rcb(pts, w, 7, 0.02)
    finite = np.isfinite(pts).all(axis=1)
    assert (ref[finite] == got[finite]).mean() > 0.5


def test_wide_negative_and_zero_weights(coupe, oracle_mod):
    rng = np.random.default_rng(22)
    pts = rng.random((60000, 3))
    w = rng.integers(-(1 << 40), 1 << 40, size=len(pts), dtype=np.int64)
    w[::7] = 0
    _check(coupe, oracle_mod, pts, w, 8, 0.01)
    w2 = np.zeros(len(pts), dtype=np.int64)  # sum 0: imbalance is NaN
    _check(coupe, oracle_mod, pts, w2, 5, 0.01)


def test_int32_wraparound(coupe, oracle_mod):
    """c_int weights whose sums overflow 32 bits wrap like release-built Rust."""
    rng = np.random.default_rng(23)
    pts = rng.random((80000, 2))
    w = rng.integers(1 << 28, (1 << 31) - 1, size=len(pts), dtype=np.int32)
    _check(coupe, oracle_mod, pts, w, 6, 0.05)


@pytest.mark.parametrize("mode", ["ref32", "f64", "f32key_f64band"])
def test_16bit_weight_copy_boundary(coupe, oracle_mod, mode):
    """Integer weights in [0, 2^16) run the level loop on a 16-bit copy: the
    largest such weight, one past it, odd segment offsets, and c_int sums that
    still wrap at 32 bits."""
    rng = np.random.default_rng(25)
    pts = rng.random((100_003, 3))
    for top in (65535, 65536):
        w = rng.integers(0, top + 1, size=len(pts), dtype=np.int64)
        w[::5] = top
        _check(coupe, oracle_mod, pts, w, 9, 0.01, mode)
    w32 = np.full(len(pts), 65535, dtype=np.int32)  # total 6.5e9: wraps in i32
    w32[::3] = 1
    _check(coupe, oracle_mod, pts, w32, 7, 0.02, mode)


def test_f64_weights_wide_range(coupe, oracle_mod):
    rng = np.random.default_rng(24)
    pts = rng.random((50000, 3))
    w = np.exp(rng.uniform(-30, 30, size=len(pts)))
    w[::13] *= -1.0
    for mode in ("ref32", "f64"):
        _check(coupe, oracle_mod, pts, w, 7, 0.01, mode)


def test_f64_weights_close_to_sequential_sums(coupe, oracle_mod):
    """Against the oracle's sequential f64 sums (the reference's arithmetic up
    to summation order): nearly all ids agree."""
    rng = np.random.default_rng(25)
    pts = rng.random((200000, 3))
    w = rng.lognormal(0.0, 1.0, size=len(pts))
    want, _ = oracle_mod.rcb(pts, w, 10, 0.01, fsum=oracle_mod.FSUM_SEQ)
    got = _gpu(coupe, pts, w, 10, 0.01)
    assert (want == got).mean() >= 0.9999


def test_iter_count_zero(coupe):
    pts = np.random.default_rng(1).random((1000, 2))
    got = _gpu(coupe, pts, np.ones(1000, np.int64), 0, 0.05)
    assert (got == 0).all()


def test_rib_with_given_matrix(coupe, oracle_mod):
    """Rib given the same basis change: bit-identical ids."""
    torch = pytest.importorskip("torch")
    from coupe_gb300 import workloads
    pts, w, _ = workloads.hex_mesh_rib(side=48, seed=5)
    M = oracle_mod.rib_matrix(pts)
    want, _ = oracle_mod.rib(pts, w, 8, 0.01, matrix=M)
    d_pts = torch.from_numpy(pts).cuda()
    d_w = torch.from_numpy(w).cuda()
    part = torch.empty(len(pts), dtype=torch.int64, device="cuda")
    coupe.rcb_device(part, d_pts, d_w, 8, 0.01, matrix=M)
    got = part.cpu().numpy().view(np.uint64)
    assert (want == got).all()


@pytest.mark.parametrize("case", ["grid", "gauss"])
def test_rib_2d_with_given_matrix(coupe, oracle_mod, case):
    """2D Rib given the same basis change: REF32 ids equal the oracle's and
    the band form's equal F64's (the f32-pair basis change of k_convert, a
    rotated grid in index order included)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    if case == "grid":
        g = np.arange(300) + 0.5
        x, y = np.meshgrid(g, g * 10, indexing="ij")
        th = 0.7
        rot = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
        pts = np.stack([x.ravel(), y.ravel()], 1) @ rot.T
    else:
        pts = rng.standard_normal((100_000, 2)) * [100.0, 3.0] + rng.standard_normal(2) * 50
    w = rng.integers(1, 100, len(pts)).astype(np.int64)
    M = oracle_mod.rib_matrix(pts)
    want, _ = oracle_mod.rib(pts, w, 7, 0.01, matrix=M)
    d_pts, d_w = torch.from_numpy(pts).cuda(), torch.from_numpy(w).cuda()
    got = {}
    for mode in ("ref32", "f64", "f32key_f64band"):
        part = torch.empty(len(pts), dtype=torch.int64, device="cuda")
        coupe.rcb_device(part, d_pts, d_w, 7, 0.01, matrix=M, mode=mode)
        got[mode] = part.cpu().numpy().view(np.uint64)
    assert (want == got["ref32"]).all()
    assert (got["f64"] == got["f32key_f64band"]).all()


def test_rib_matrix_matches_oracle(coupe, oracle_mod):
    torch = pytest.importorskip("torch")
    from coupe_gb300 import workloads
    pts, _, _ = workloads.hex_mesh_rib(side=40, seed=6)
    M_o = oracle_mod.rib_matrix(pts)
    M_g = coupe.rib_matrix_device(torch.from_numpy(pts).cuda())
    assert np.allclose(M_g, M_o, rtol=1e-9, atol=1e-12)


def test_rib_end_to_end(coupe, oracle_mod):
    from coupe_gb300 import workloads
    pts, w, _ = workloads.hex_mesh_rib(side=40, seed=7)
    want, _ = oracle_mod.rib(pts, w, 8, 0.01)
    got = _gpu(coupe, pts, w, 8, 0.01, rib=True)
    assert (want == got).mean() >= 0.9999


@pytest.mark.parametrize("knobs", [{"force_index_path": 1}, {"max_nbk": 3}, {"max_nbk": 1}, {"max_nbk": 8},
                                   {"reorder_chunks_per_cta": 4}, {"reorder_chunks_per_cta": 64},
                                   {"max_nbk": 5, "reorder_chunks_per_cta": 3},
                                   {"force_index_path": 1, "reorder_chunks_per_cta": 7},
                                   {"hist_ctas_per_sm": 1}, {"hist_ctas_per_sm": 2, "max_nbk": 9},
                                   {"sync_levels": 1}, {"sync_levels": 1, "max_nbk": 2}, {"max_nbk": 2},
                                   {"reorder_kernel": 1}, {"reorder_kernel": 2}, {"hist_waves": 3},
                                   {"reorder_kernel": 1, "force_index_path": 1}, {"reorder_kernel": 2, "force_index_path": 1}])
def test_scheduling_knobs_do_not_change_ids(coupe, oracle_mod, knobs):
    """Part ids through the index path, fewer bisection steps per pass and
    other chunkings equal the oracle's."""
    from coupe_gb300 import workloads
    pts, w, cfg = workloads.gaussian_mixture3d(n=120_000, seed=9)
    want, _ = oracle_mod.rcb(pts, w, 9, 0.01)
    old = {k: coupe.get_option(k) for k in knobs}
    try:
        for k, v in knobs.items():
            coupe.set_option(k, v)
        for mode, om in (("ref32", 0), ("f64", 1), ("f32key_f64band", 1)):
            want, _ = oracle_mod.rcb(pts, w, 9, 0.01, mode=om)
            got = _gpu(coupe, pts, w, 9, 0.01, mode=mode)
            assert (want == got).all()
        # deep tree on the same path
        p2, w2 = _make(3000, 2, "i64", 11)
        want2, _ = oracle_mod.rcb(p2, w2, 14, 0.05)
        assert (want2 == _gpu(coupe, p2, w2, 14, 0.05)).all()
    finally:
        for k, v in old.items():
            coupe.set_option(k, v)


@pytest.mark.parametrize("mode", ["ref32", "f64", "f32key_f64band"])
def test_full_size_repeatable(coupe, oracle_mod, mode):
    """16.8 M points, 1024 parts (the benchmark workload): equal to the
    oracle once, then 40 device-resident runs in a row give the same ids and
    raise no device check (look-back, scatter bounds, tile permutation)."""
    torch = pytest.importorskip("torch")
    import os
    from coupe_gb300 import workloads
    pts, w, cfg = workloads.gaussian_mixture3d(n=16_777_216, seed=0)
    want, _ = oracle_mod.rcb(pts, w, 10, 0.01, mode=_oracle_mode(mode), threads=os.cpu_count() or 1)
    dp = torch.from_numpy(pts).cuda()
    dw = torch.from_numpy(w).cuda()
    part = torch.empty(len(pts), dtype=torch.int64, device="cuda")
    coupe.rcb_device(part, dp, dw, 10, 0.01, mode=mode)
    first = part.clone()
    assert (part.cpu().numpy().astype(np.uint64) == want).all()
    for _ in range(40):
        part.fill_(-1)
        coupe.rcb_device(part, dp, dw, 10, 0.01, mode=mode)
        assert torch.equal(part, first)


@pytest.mark.parametrize("dim", [2, 3])
def test_band_inside_one_f32_interval(coupe, oracle_mod, dim):
    """Band form: coordinates packed inside one or two f32 rounding intervals,
    so that every cut of the first axis lies in the band: the f64 coordinate
    decides every bin, every side and the exact minima of the stop test.  The
    ids equal the F64 form's (the oracle's f64 mode)."""
    rng = np.random.default_rng(31 + dim)
    n = 60_000
    pts = rng.random((n, dim))
    pts[:, 0] = 1.0 + rng.integers(0, 1 << 21, size=n) * 2.0 ** -44  # within 2^-23 of 1
    pts[::97, 0] = 1.0 + 2.0 ** -24  # the halfway point between two floats
    w = rng.integers(1, 50, size=n, dtype=np.int64)
    for iters, tol in ((6, 0.01), (9, 0.001)):
        _check(coupe, oracle_mod, pts, w, iters, tol, "f32key_f64band")
    st = coupe.last_stats()
    assert st["mode"] == 2


def test_rib_band_equals_f64(coupe):
    """Rib in the band form gathers the rotated f64 coordinate exactly as the
    conversion computed it: the ids equal the F64 form's."""
    from coupe_gb300 import workloads
    pts, w, _ = workloads.hex_mesh_rib(side=40, seed=8)
    a = _gpu(coupe, pts, w, 9, 0.01, mode="f64", rib=True)
    b = _gpu(coupe, pts, w, 9, 0.01, mode="f32key_f64band", rib=True)
    assert (a == b).all()


def test_key_conversion_is_ieee_rne(coupe):
    """The engine's integer f64 -> f32 conversion equals IEEE round-to-nearest-
    even (numpy's cast) on random bit patterns, the f32 range edges, halfway
    cases and the special values."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(30)
    bits = [rng.integers(0, 2**64, size=4_000_000, dtype=np.uint64)]
    e = rng.integers(896 - 40, 1151 + 40, size=2_000_000, dtype=np.uint64)
    frac = rng.integers(0, 2**52, size=len(e), dtype=np.uint64)
    sign = rng.integers(0, 2, size=len(e), dtype=np.uint64) << np.uint64(63)
    bits.append(sign | (e << np.uint64(52)) | frac)
    half = (sign | (e << np.uint64(52)) | (frac & ~np.uint64((1 << 29) - 1)) | np.uint64(1 << 28))
    bits += [half, half - np.uint64(1), half + np.uint64(1)]
    bits.append(np.array([0, 1 << 63, 0x7FF0 << 48, 0xFFF0 << 48, 0x7FF8 << 48, 1, 0x47EFFFFFE0000000,
                          0x47EFFFFFEFFFFFFF, 0x47EFFFFFF0000000, 0x36A0000000000000, 0x3690000000000000,
                          0x3690000000000001, 0x380FFFFFE0000000], dtype=np.uint64))
    b = np.concatenate(bits)
    x = b.view(np.float64)
    with np.errstate(over="ignore", invalid="ignore"):
        want = x.astype(np.float32)
    d_in = torch.from_numpy(x.copy()).cuda()
    d_out = torch.empty(len(x), dtype=torch.float32, device="cuda")
    L = coupe.lib()
    stream = torch.cuda.current_stream().cuda_stream
    assert L.coupe_gpu_f64_to_f32(d_in.data_ptr(), d_out.data_ptr(), len(x), stream) == 0
    got = d_out.cpu().numpy()
    nan = np.isnan(want)
    assert (np.isnan(got) == nan).all()
    assert (got[~nan].view(np.uint32) == want[~nan].view(np.uint32)).all()


# ---------------------------------------------------------------------------
# f64 weights: bins of truncated fixed-point weights, exact replays
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("mode", ["ref32", "f64", "f32key_f64band"])
def test_f64_weights_exact_bins_equal_truncated_bins(coupe, oracle_mod, mode):
    """The f64 random cases with the histograms forced to exact fixed-point
    sums give the same ids as the default truncated bins (and the oracle)."""
    cases = [c for c in CASES if c[2] == "f64"]
    try:
        for n, dim, wk, iters, tol, seed in cases:
            pts, w = _make(n, dim, wk, seed)
            want, _ = oracle_mod.rcb(pts, w, iters, tol, mode=_oracle_mode(mode))
            coupe.set_option("exact_f64_hist", 1)
            exact = _gpu(coupe, pts, w, iters, tol, mode=mode)
            assert coupe.last_stats()["weight_rechecks"] == 0
            coupe.set_option("exact_f64_hist", 0)
            trunc = _gpu(coupe, pts, w, iters, tol, mode=mode)
            assert np.array_equal(exact, want) and np.array_equal(trunc, want), (n, dim, iters)
    finally:
        coupe.set_option("exact_f64_hist", 0)


@pytest.mark.parametrize("mode", ["ref32", "f32key_f64band"])
@pytest.mark.parametrize("tol", [0.0, 1e-7])
def test_f64_weights_undecided_steps_replay_exactly(coupe, oracle_mod, mode, tol):
    """Tolerances 0 and 1e-7: weight_left is compared with sum/2 closer than
    the truncated bins can tell, so splits replay steps from exact bins
    (weight_rechecks > 0); the ids still equal the oracle's."""
    rng = np.random.default_rng(77)
    n = 300_000
    pts = rng.random((n, 3))
    w = rng.lognormal(0.0, 2.0, n)
    want, _ = oracle_mod.rcb(pts, w, 8, tol, mode=_oracle_mode(mode))
    got = _gpu(coupe, pts, w, 8, tol, mode=mode)
    assert coupe.last_stats()["weight_rechecks"] > 0
    assert np.array_equal(got, want)


def test_f64_weights_negative_use_exact_bins(coupe, oracle_mod):
    """Negative f64 weights have no truncated bins (every pass is exact)."""
    rng = np.random.default_rng(78)
    pts = rng.random((200_000, 2))
    w = rng.normal(1.0, 3.0, len(pts))
    for mode, om in (("f64", 1), ("f32key_f64band", 1), ("ref32", 0)):
        want, _ = oracle_mod.rcb(pts, w, 7, 0.01, mode=om)
        got = _gpu(coupe, pts, w, 7, 0.01, mode=mode)
        assert coupe.last_stats()["weight_rechecks"] == 0
        assert np.array_equal(got, want)


@pytest.mark.parametrize("mode", ["ref32", "f64", "f32key_f64band"])
@pytest.mark.parametrize("nbk,exact", [(6, 0), (7, 1), (4, 0)])
def test_small_segments_binned_per_warp(coupe, oracle_mod, mode, nbk, exact):
    """With at most 128 bins a pass, segments of up to 4096 items are binned
    one per warp: ids equal the oracle's, for int64 and f64 weights, NaN keys
    and keys piled on a few values (band items)."""
    rng = np.random.default_rng(90 + nbk)
    n = 150_000
    pts = rng.random((n, 3))
    pts[::7, 0] = 0.5
    pts[::11, 1] = np.round(pts[::11, 1], 2)
    pts[5::997, 2] = np.nan
    try:
        coupe.set_option("max_nbk", nbk)
        coupe.set_option("exact_f64_hist", exact)
        for w in (rng.integers(1, 50, n, dtype=np.int64), rng.lognormal(0.0, 1.0, n)):
            want, _ = oracle_mod.rcb(pts, w, 11, 0.01, mode=_oracle_mode(mode) | oracle_mod.NAN_RIGHT)
            got = _gpu(coupe, pts, w, 11, 0.01, mode=mode)
            assert np.array_equal(got, want)
    finally:
        coupe.set_option("max_nbk", 10)
        coupe.set_option("exact_f64_hist", 0)


def test_pinned_host_buffers(coupe, oracle_mod):
    """Host calls with pinned (page-locked) buffers: the weights upload
    overlaps the key conversion and the ids are written straight into the
    pinned id buffer (or copied after, on the index path).  Same ids as with
    pageable buffers and as the oracle."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(91)
    n = 300_000
    for dim, wk in ((3, "i64"), (2, "f64")):
        pts, w = _make(n, dim, wk, 91 + dim)
        pp = torch.from_numpy(pts).pin_memory().numpy()
        pw = torch.from_numpy(w).pin_memory().numpy()
        for knobs in ({}, {"force_index_path": 1}):
            old = {k: coupe.get_option(k) for k in knobs}
            try:
                for k, v in knobs.items():
                    coupe.set_option(k, v)
                for mode in ("ref32", "f32key_f64band"):
                    want, _ = oracle_mod.rcb(pts, w, 9, 0.01, mode=_oracle_mode(mode))
                    ids = torch.zeros(n, dtype=torch.int64).pin_memory().numpy().view(np.uint64)
                    ids[:] = 12345
                    coupe.Rcb(iter_count=9, tolerance=0.01, mode=mode).partition(ids, (pp, pw))
                    assert np.array_equal(ids, want), (dim, wk, knobs, mode)
                    ids2 = torch.zeros(n, dtype=torch.int64).pin_memory().numpy().view(np.uint64)
                    coupe.Rib(iter_count=5, tolerance=0.02, mode=mode).partition(ids2, (pp, pw))
                    ref = np.zeros(n, dtype=np.uint64)
                    coupe.Rib(iter_count=5, tolerance=0.02, mode=mode).partition(ref, (pts, w))
                    assert np.array_equal(ids2, ref)
            finally:
                for k, v in old.items():
                    coupe.set_option(k, v)


@pytest.mark.parametrize("mode", ["ref32", "f32key_f64band"])
def test_queued_run_waits_once(coupe, oracle_mod, mode):
    """A run is queued whole: the host waits for the 16-bit weight check and
    for the end (2 synchronisations), against one per level with
    sync_levels; a split needing more than two histogram passes (max_nbk 2)
    halts the queue and the host finishes level by level.  Same ids."""
    from coupe_gb300 import workloads
    pts, w, _ = workloads.gaussian_mixture3d(n=200_000, seed=12)
    om = oracle_mod.REF32 if mode == "ref32" else oracle_mod.F64
    want, _ = oracle_mod.rcb(pts, w, 9, 0.01, mode=om)
    assert (_gpu(coupe, pts, w, 9, 0.01, mode=mode) == want).all()
    assert coupe.last_stats()["host_syncs"] <= 2
    old = {k: coupe.get_option(k) for k in ("sync_levels", "max_nbk")}
    try:
        coupe.set_option("sync_levels", 1)
        assert (_gpu(coupe, pts, w, 9, 0.01, mode=mode) == want).all()
        assert coupe.last_stats()["host_syncs"] >= 9
        coupe.set_option("sync_levels", 0)
        coupe.set_option("max_nbk", 2)
        assert (_gpu(coupe, pts, w, 9, 0.01, mode=mode) == want).all()
        assert coupe.last_stats()["host_syncs"] > 2  # halted, then level by level
    finally:
        for k, v in old.items():
            coupe.set_option(k, v)
