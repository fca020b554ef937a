"""CPU checks of the seeded workload generators the benchmark and the GPU
tests use (the reference measures on no public dataset, so these define the
benchmark inputs), and of the oracle's per-set helper."""
import numpy as np

from coupe_gb300 import workloads


def test_gaussian_mixture_is_seeded():
    a, wa, ca = workloads.gaussian_mixture3d(n=10_000, seed=3)
    b, wb, cb = workloads.gaussian_mixture3d(n=10_000, seed=3)
    assert np.array_equal(a, b) and np.array_equal(wa, wb)
    assert a.shape == (10_000, 3) and wa.dtype == np.int64
    assert wa.min() >= 1 and wa.max() <= 100
    assert ca["iter_count"] == 10 and ca["tolerance"] == 0.01


def test_planes_workload_shape():
    p, w, c = workloads.planes3d_lognormal(n=200_000, seed=1)
    on = np.isin(p[:, 0], [0.25, 0.5, 0.75])
    assert 0.04 < on.mean() < 0.06  # 5 % of the points on the planes
    assert w.dtype == np.float64 and (w > 0).all()
    assert c["iter_count"] == 12 and c["tolerance"] == 0.005


def test_batched_groups_match_sets():
    sets = workloads.batched_sets(n_sets=24, seed=5, total=200_000)
    groups = workloads.batched_groups(n_sets=24, seed=5, total=200_000)
    assert set(groups) == {2, 3}
    for d, (pts, w, off, it, ids) in groups.items():
        assert off[0] == 0 and off[-1] == len(pts) == len(w)
        for j, s in enumerate(ids):
            p, ws, i = sets[s]
            assert p.shape[1] == d
            assert np.array_equal(pts[off[j]:off[j + 1]], p)
            assert np.array_equal(w[off[j]:off[j + 1]], ws)
            assert it[j] == i and 1 <= i <= 8


def test_hex_mesh_rotation():
    p, w, c = workloads.hex_mesh_rib(side=8, seed=2)
    assert p.shape == (512, 3)
    # a rotation keeps the distances between cells
    q = np.stack(np.meshgrid(np.arange(8) + 0.5, (np.arange(8) + 0.5) * 10, (np.arange(8) + 0.5) * 100,
                             indexing="ij"), axis=-1).reshape(-1, 3)
    d1 = np.linalg.norm(p[1:] - p[:-1], axis=1)
    d2 = np.linalg.norm(q[1:] - q[:-1], axis=1)
    assert np.allclose(d1, d2)
    assert (w >= 1000.0).all() and (w < 2000.0).all()


def test_oracle_sets_equal_separate_runs(oracle_mod):
    rng = np.random.default_rng(4)
    sizes = [0, 5, 300, 1, 2000]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    pts = rng.random((int(off[-1]), 2))
    w = rng.integers(1, 9, int(off[-1]), dtype=np.int64)
    it = np.array([3, 2, 4, 0, 5], dtype=np.uint32)
    got = oracle_mod.rcb_sets(pts, w, off, it, 0.05)
    for k in range(len(sizes)):
        a, b = int(off[k]), int(off[k + 1])
        if b > a:
            want, _ = oracle_mod.rcb(pts[a:b], w[a:b], int(it[k]), 0.05)
            assert np.array_equal(got[a:b], want)
