"""The batched form (coupe_gpu_rcb_batched): many independent point sets in
one run.  Each set's ids must equal those of a run of that set alone: the
oracle per set (bit-identical, integer and f64 weights alike, since each set
keeps its own fixed-point scale), and the library's own one-set entry point.
"""
import numpy as np
import pytest

from coupe_gb300 import workloads

pytestmark = pytest.mark.gpu

MODES = ["ref32", "f64", "f32key_f64band"]


def _oracle_mode(mode):
    return 1 if mode in ("f64", "f32key_f64band") else 0


def _sets(rng, sizes, dim, wk, iters):
    off = np.zeros(len(sizes) + 1, dtype=np.uint64)
    np.cumsum(np.asarray(sizes, dtype=np.uint64), out=off[1:])
    n = int(off[-1])
    pts = np.empty((n, dim))
    for k in range(len(sizes)):
        a, b = int(off[k]), int(off[k + 1])
        lo = rng.uniform(-50, 50, dim)
        pts[a:b] = lo + rng.random((b - a, dim)) * rng.uniform(0.5, 80.0, dim)
        if b - a > 10:
            pts[a:a + (b - a) // 8] = np.round(pts[a:a + (b - a) // 8], 1)  # ties
    if wk == "i64":
        w = rng.integers(1, 100, n, dtype=np.int64)
    elif wk == "i32":
        w = rng.integers(1, 100, n, dtype=np.int32)
    elif wk == "wide":
        w = rng.integers(-5, 1 << 20, n, dtype=np.int64)
    else:
        w = rng.lognormal(0.0, 1.0, n) * np.repeat(rng.lognormal(0.0, 3.0, len(sizes)), sizes)
    return pts, w, off, np.asarray(iters, dtype=np.uint32)


def _gpu(coupe, torch, pts, w, off, iters, tol, mode):
    dp = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    dw = torch.from_numpy(np.ascontiguousarray(w)).cuda()
    ids = torch.full((len(pts),), -1, dtype=torch.int64, device="cuda")
    coupe.rcb_batched_device(ids, dp, dw, off, iters, tol, mode=mode)
    return ids.cpu().numpy().astype(np.uint64)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("dim,wk,seed", [(2, "i64", 1), (3, "i32", 2), (3, "f64", 3), (2, "wide", 4), (3, "i64", 5)])
def test_batched_equals_oracle_per_set(coupe, oracle_mod, dim, wk, seed, mode):
    """Ragged sets: empty, single points, tiny and larger sets; iter_count 0
    to 9 per set (sets that stop early drop out of later levels)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(seed)
    sizes = [0, 1, 2, 7, 3000, 0, 50_000, 1, 120_000, 999, 17, 40_000, 0, 4096, 65_537, 5]
    sizes += [int(x) for x in rng.integers(1, 30_000, 24)]
    iters = rng.integers(0, 10, len(sizes))
    iters[4] = 0  # a non-empty set with iter_count 0: id 0 everywhere
    iters[6] = 9
    pts, w, off, it = _sets(rng, sizes, dim, wk, iters)
    tol = 0.01
    want = oracle_mod.rcb_sets(pts, w, off, it, tol, mode=_oracle_mode(mode), fsum=oracle_mod.FSUM_FIXED)
    got = _gpu(coupe, torch, pts, w, off, it, tol, mode)
    bad = np.nonzero(want != got)[0]
    assert len(bad) == 0, "%d ids differ, first at %d" % (len(bad), bad[0])


@pytest.mark.parametrize("mode", MODES)
def test_batched_equals_one_set_runs(coupe, mode):
    """Against coupe_gpu_rcb_device on each set (larger sets, f64 weights)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    sizes = [int(x) for x in rng.integers(100_000, 700_000, 12)]
    iters = rng.integers(1, 9, len(sizes))
    pts, w, off, it = _sets(rng, sizes, 3, "f64", iters)
    got = _gpu(coupe, torch, pts, w, off, it, 0.005, mode)
    for k in range(len(sizes)):
        a, b = int(off[k]), int(off[k + 1])
        ids = torch.zeros(b - a, dtype=torch.int64, device="cuda")
        coupe.rcb_device(ids, torch.from_numpy(pts[a:b]).cuda(), torch.from_numpy(w[a:b]).cuda(), int(it[k]),
                         0.005, mode=mode)
        assert np.array_equal(ids.cpu().numpy().astype(np.uint64), got[a:b]), "set %d" % k


@pytest.mark.parametrize("mode", MODES)
def test_batched_workload_shape(coupe, oracle_mod, mode):
    """The batched benchmark's generator at 1/40 of its size (512 sets,
    5e6 points), both dimension groups, against the oracle per set."""
    torch = pytest.importorskip("torch")
    groups = workloads.batched_groups(n_sets=512, seed=3, total=5_000_000)
    for dim, (pts, w, off, it, _) in groups.items():
        want = oracle_mod.rcb_sets(pts, w, off, it, 0.01, mode=_oracle_mode(mode), threads=0)
        got = _gpu(coupe, torch, pts, w, off, it, 0.01, mode)
        assert np.array_equal(want, got), "dim %d: %d ids differ" % (dim, int((want != got).sum()))


def test_batched_edge_cases(coupe, oracle_mod):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    # every set empty but one; every iter_count 0; one point per set
    for sizes, iters in [([0, 0, 5000, 0], [3, 3, 4, 3]), ([10, 20, 30], [0, 0, 0]), ([1] * 300, [5] * 300),
                         ([3000, 3000], [1, 1]), ([2000] * 3, [9, 0, 9])]:
        pts, w, off, it = _sets(rng, sizes, 2, "i64", iters)
        want = oracle_mod.rcb_sets(pts, w, off, it, 0.05)
        got = _gpu(coupe, torch, pts, w, off, it, 0.05, "ref32")
        assert np.array_equal(want, got), (sizes, iters)
    # identical points within a set, NaN coordinates, repeated calls
    pts, w, off, it = _sets(rng, [5000, 7000, 3000], 3, "i64", [4, 6, 2])
    pts[0:5000] = 1.5
    pts[6000:6100, 1] = np.nan
    want = oracle_mod.rcb_sets(pts, w, off, it, 0.01, mode=oracle_mod.F64 | oracle_mod.NAN_RIGHT)
    for _ in range(2):
        got = _gpu(coupe, torch, pts, w, off, it, 0.01, "f64")
        assert np.array_equal(want, got)


def test_batched_matches_after_other_sizes(coupe, oracle_mod):
    """A small batch after a large one-set run on the same device (workspace
    reuse), then a large batch."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(12)
    big = torch.from_numpy(rng.random((2_000_000, 3))).cuda()
    ids = torch.zeros(2_000_000, dtype=torch.int64, device="cuda")
    coupe.rcb_device(ids, big, torch.ones(2_000_000, dtype=torch.int64, device="cuda"), 10, 0.01)
    for sizes in ([300, 5, 4000], [int(x) for x in rng.integers(1000, 200_000, 40)]):
        iters = rng.integers(1, 9, len(sizes))
        pts, w, off, it = _sets(rng, sizes, 3, "i64", iters)
        want = oracle_mod.rcb_sets(pts, w, off, it, 0.01, threads=0)
        assert np.array_equal(want, _gpu(coupe, torch, pts, w, off, it, 0.01, "ref32"))


def test_autotune_keeps_ids(coupe, oracle_mod):
    """The autotuner picks one of its candidate schedules; the ids under it
    are those of the default schedule (and of the oracle)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    sizes = [int(x) for x in rng.integers(5_000, 300_000, 30)]
    iters = rng.integers(1, 9, len(sizes))
    pts, w, off, it = _sets(rng, sizes, 3, "i64", iters)
    want = oracle_mod.rcb_sets(pts, w, off, it, 0.01, mode=1, threads=0)
    names = ("max_nbk", "hist_ctas_per_sm", "reorder_chunks_per_cta", "hist_waves")
    keep = {k: coupe.get_option(k) for k in names + ("autotune_cache",)}
    try:
        coupe.set_option("autotune_cache", 0)  # time the candidates here
        dp = torch.from_numpy(pts).cuda()
        dw = torch.from_numpy(w).cuda()
        ids = torch.zeros(len(pts), dtype=torch.int64, device="cuda")
        best = coupe.autotune_device(ids, dp, dw, off, it, 0.01, mode="f32key_f64band", repeats=1)
        assert best["max_nbk"] in (6, 7, 8, 9, 10) and best["hist_ctas_per_sm"] in (0, 2, 3)
        assert best["reorder_chunks_per_cta"] in (1, 2) and best["hist_waves"] in (1, 2) and best["device_ms"] > 0
        assert {k: coupe.get_option(k) for k in names} == {k: best[k] for k in names}
        assert np.array_equal(ids.cpu().numpy().astype(np.uint64), want)
        assert np.array_equal(_gpu(coupe, torch, pts, w, off, it, 0.01, "f32key_f64band"), want)
    finally:
        for k, v in keep.items():
            coupe.set_option(k, v)


def test_autotune_keeps_its_choice_per_workload_class(coupe, tmp_path, monkeypatch):
    """A second call for the same workload class applies the kept schedule
    without running; the choice is written to COUPE_GPU_TUNE_CACHE."""
    torch = pytest.importorskip("torch")
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("COUPE_GPU_TUNE_CACHE", str(cache))
    rng = np.random.default_rng(22)
    sizes = [int(x) for x in rng.integers(5_000, 50_000, 9)]
    iters = np.full(len(sizes), 7)
    pts, w, off, it = _sets(rng, sizes, 2, "i32", iters)
    names = ("max_nbk", "hist_ctas_per_sm", "reorder_chunks_per_cta", "hist_waves")
    keep = {k: coupe.get_option(k) for k in names + ("autotune_cache",)}
    try:
        coupe.set_option("autotune_cache", 1)
        dp = torch.from_numpy(pts).cuda()
        dw = torch.from_numpy(w).cuda()
        ids = torch.zeros(len(pts), dtype=torch.int64, device="cuda")
        first = coupe.autotune_device(ids, dp, dw, off, it, 0.02, mode="ref32", repeats=1)
        for k, v in keep.items():  # another schedule in force
            coupe.set_option(k, v)
        coupe.set_option("autotune_cache", 1)
        ids2 = torch.full((len(pts),), 7, dtype=torch.int64, device="cuda")
        again = coupe.autotune_device(ids2, dp, dw, off, it, 0.02, mode="ref32", repeats=1)
        assert again == first
        assert {k: coupe.get_option(k) for k in names} == {k: first[k] for k in names}
        assert (ids2 == 7).all()  # nothing ran
        lines = cache.read_text().split("\n")
        assert any(l.startswith("n2^") and l.split()[1] == str(first["max_nbk"]) for l in lines)
    finally:
        for k, v in keep.items():
            coupe.set_option(k, v)
