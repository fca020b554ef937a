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


def _main(argv=None):
    """Runs one workload through the device API a few times and prints the
    library's per-kernel CUDA-event times (the command profiles are taken
    with):

        python -m coupe_gb300.workloads gauss16M --mode f32key_f64band --runs 3
        python -m coupe_gb300.workloads planes67M --points 16777216
        python -m coupe_gb300.workloads hexrib134M --side 256
        python -m coupe_gb300.workloads batched4096 --total 50000000
        python -m coupe_gb300.workloads uniform1M
    """
    import argparse
    import json

    import torch

    import coupe_gb300 as coupe
    ap = argparse.ArgumentParser(prog="python -m coupe_gb300.workloads")
    ap.add_argument("workload", choices=["uniform1M", "gauss16M", "planes67M", "batched4096", "hexrib134M"])
    ap.add_argument("--mode", default="f32key_f64band", choices=sorted(coupe.MODES))
    ap.add_argument("--runs", type=int, default=3)
    ap.add_argument("--points", type=int, default=None, help="points (uniform1M, gauss16M, planes67M)")
    ap.add_argument("--side", type=int, default=512, help="hex mesh side (hexrib134M)")
    ap.add_argument("--sets", type=int, default=4096, help="sets (batched4096)")
    ap.add_argument("--total", type=int, default=200_000_000, help="about this many points (batched4096)")
    ap.add_argument("--option", action="append", default=[], metavar="NAME=VALUE",
                    help="a library option (coupe_gpu_set_option), e.g. reorder_kernel=2")
    a = ap.parse_args(argv)
    for o in a.option:
        name, value = o.split("=", 1)
        coupe.set_option(name, int(value))
    dev = torch.device("cuda", 0)
    kw = {} if a.points is None else {"n": a.points}
    if a.workload == "batched4096":
        groups = batched_groups(a.sets, 0, a.total)
        calls = []
        for d, (p, w, off, it, _) in groups.items():
            dp, dw = torch.from_numpy(p).to(dev), torch.from_numpy(w).to(dev)
            out = torch.empty(len(p), dtype=torch.int64, device=dev)
            calls.append(lambda out=out, dp=dp, dw=dw, off=off, it=it:
                         coupe.rcb_batched_device(out, dp, dw, off, it, 0.01, mode=a.mode))
        n = sum(len(g[0]) for g in groups.values())
    else:
        gen = {"uniform1M": uniform2d_unit, "gauss16M": gaussian_mixture3d, "planes67M": planes3d_lognormal}
        if a.workload == "hexrib134M":
            p, w, c = hex_mesh_rib(side=a.side)
        else:
            p, w, c = gen[a.workload](**kw)
        dp, dw = torch.from_numpy(p).to(dev), torch.from_numpy(w).to(dev)
        out = torch.empty(len(p), dtype=torch.int64, device=dev)
        f = coupe.rib_device if a.workload == "hexrib134M" else coupe.rcb_device
        calls = [lambda: f(out, dp, dw, c["iter_count"], c["tolerance"], mode=a.mode)]
        n = len(p)
    for call in calls:  # warm-up (workspace, autotune cache)
        call()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(a.runs):
        for call in calls:
            call()
    ev1.record()
    torch.cuda.synchronize()
    coupe.profile(True)
    for _ in range(a.runs):
        for call in calls:
            call()
    torch.cuda.synchronize()
    prof = coupe.profile_read()
    coupe.profile(False)
    print(json.dumps({"workload": a.workload, "points": n, "mode": a.mode, "runs": a.runs,
                      "ms_per_run": round(ev0.elapsed_time(ev1) / a.runs, 4),
                      "kernels": {k: {"launches_per_run": v["launches"] / a.runs,
                                      "us_per_run": round(1e3 * v["ms"] / a.runs, 1),
                                      "algorithmic_bytes_per_launch": v["bytes"] // max(1, v["launches"])}
                                  for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])}}))


if __name__ == "__main__":
    _main()
