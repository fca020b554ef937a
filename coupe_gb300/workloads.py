"""Seeded synthetic inputs for the five benchmark configurations.

The reference measures on no public dataset, so these generators are the
whole benchmark: AoS float64 points exactly as the C ABI receives them, and
weights of the stated type.  numpy's PCG64 gives the same numbers on x86_64
and aarch64.
"""
import numpy as np


def uniform2d_unit(n=1_000_000, seed=0):
    """1: n 2D points U[0,1)^2, unit int64 weights (iter_count 3, tolerance 0.05)."""
    rng = np.random.default_rng(seed)
    pts = rng.random((n, 2))
    w = np.ones(n, dtype=np.int64)
    return pts, w, dict(iter_count=3, tolerance=0.05, name="uniform2d_1M_iter3")


def gaussian_mixture3d(n=16_777_216, seed=0, clusters=32):
    """2: n 3D points from a mixture of 32 isotropic Gaussians (centres
    U[0,100]^3, sigma U[0.5,5], equal mixture weights); int64 weights U{1..100}
    (iter_count 10 -> 1024 parts, tolerance 0.01)."""
    rng = np.random.default_rng(seed)
    centres = rng.random((clusters, 3)) * 100.0
    sigma = 0.5 + rng.random(clusters) * 4.5
    comp = rng.integers(0, clusters, size=n)
    pts = rng.standard_normal((n, 3))
    pts *= sigma[comp, None]
    pts += centres[comp]
    w = rng.integers(1, 101, size=n, dtype=np.int64)
    return pts, w, dict(iter_count=10, tolerance=0.01, name="gauss3d_16M_1024parts")


def planes3d_lognormal(n=67_108_864, seed=0):
    """3: n 3D points U[0,1)^3, 5% with x moved onto {0.25, 0.5, 0.75};
    float64 weights lognormal(0, 1) (iter_count 12 -> 4096 parts, tolerance 0.005)."""
    rng = np.random.default_rng(seed)
    pts = rng.random((n, 3))
    m = rng.random(n) < 0.05
    pts[m, 0] = rng.choice(np.array([0.25, 0.5, 0.75]), size=int(m.sum()))
    w = rng.lognormal(0.0, 1.0, size=n)
    return pts, w, dict(iter_count=12, tolerance=0.005, name="planes3d_67M_4096parts")


def _batched_iter(n_sets, seed, total):
    rng = np.random.default_rng(seed)
    raw = rng.lognormal(0.0, 1.0, size=n_sets)
    sizes = np.clip(raw / raw.sum() * total, 1_000, 1_000_000).astype(np.int64)
    for s in range(n_sets):
        d = 2 if s % 2 == 0 else 3
        lo = rng.random(d) * 100.0
        span = 1.0 + rng.random(d) * 99.0
        pts = lo + rng.random((int(sizes[s]), d)) * span
        w = rng.integers(1, 11, size=int(sizes[s]), dtype=np.int64)
        yield s, pts, w, int(rng.integers(1, 9))


def batched_sets(n_sets=4096, seed=0, total=200_000_000):
    """4: n_sets independent point sets, sizes lognormal clipped to
    [1e3, 1e6] scaled to about `total` points, half 2D half 3D, coordinates
    uniform in a per-set random box, int64 weights U{1..10}, iter_count
    U{1..8} per set.  Returns a list of (points, weights, iter_count)."""
    return [(p, w, it) for _, p, w, it in _batched_iter(n_sets, seed, total)]


def batched_groups(n_sets=4096, seed=0, total=200_000_000):
    """The sets of batched_sets (same values), concatenated per dimension in
    set order, as one batched call per dimension takes them:
    {dim: (points (N, dim), weights (N,), set offsets (k + 1,), iter counts
    (k,), set numbers (k,))}."""
    parts = {2: [], 3: []}
    for s, p, w, it in _batched_iter(n_sets, seed, total):
        parts[p.shape[1]].append((s, p, w, it))
    out = {}
    for d, lst in parts.items():
        if not lst:
            continue
        sizes = np.array([len(p) for _, p, _, _ in lst], dtype=np.uint64)
        off = np.zeros(len(lst) + 1, dtype=np.uint64)
        np.cumsum(sizes, out=off[1:])
        out[d] = (np.concatenate([p for _, p, _, _ in lst]), np.concatenate([w for _, _, w, _ in lst]), off,
                  np.array([it for _, _, _, it in lst], dtype=np.uint32),
                  np.array([s for s, _, _, _ in lst], dtype=np.int64))
    return out


def random_rotation(rng):
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q *= np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def hex_mesh_rib(side=512, seed=0):
    """5: centroids of a side^3 unit hex grid stretched by (1, 10, 100) and
    rotated by a seeded random rotation; float64 weights = cell volume *
    (1 + U[0,1)) (Rib, iter_count 10, tolerance 0.01)."""
    rng = np.random.default_rng(seed)
    g = (np.arange(side, dtype=np.float64) + 0.5)
    x, y, z = np.meshgrid(g, g * 10.0, g * 100.0, indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    del x, y, z
    rot = random_rotation(rng)
    pts = pts @ rot.T
    vol = 1.0 * 10.0 * 100.0
    w = vol * (1.0 + rng.random(len(pts)))
    return pts, w, dict(iter_count=10, tolerance=0.01, name="hexmesh_rib_%d^3" % side)
