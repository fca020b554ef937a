"""Float-weight parity at the sizes of the f64-weight workloads' generators.

coupe sums f64 weights in rayon's order (recursive_bisection.rs:478-520,
684); the GPU sums an order-independent 128-bit fixed point.  These tests pin
the GPU against the reference's own arithmetic — the oracle's sequential f64
sums (coupe with one rayon thread) and its chunked sums (rayon's fold per
chunk, then the reduce) — on the planes generator (f64 lognormal weights,
4096 parts) and the stretched hex-mesh Rib generator, at 4M points each, by
the criteria of oracle/float_parity.py: >= 99.99 % identical ids, no split
over the tolerance where the reference's is within it, every mismatching id
traced to a split position within one ulp (oracle/float_parity.py).  The CPU tests run the same
criteria between the oracle's fixed-point sums (which the GPU equals bit for
bit, tests/test_gpu_parity.py) and its f64 sums; the GPU tests compare the
GPU itself.
"""
import math

import numpy as np
import pytest

import float_parity as fp

N_PLANES = 1 << 22      # 4,194,304 points, planes3d_lognormal
HEX_SIDE = 160          # 4,096,000 cells, hex_mesh_rib


def _planes():
    from coupe_gb300 import workloads
    return workloads.planes3d_lognormal(n=N_PLANES, seed=1)


def _hex():
    from coupe_gb300 import workloads
    return workloads.hex_mesh_rib(side=HEX_SIDE, seed=1)


def _assert_criteria(r):
    assert r["identical"] >= 0.9999, r
    assert r["splits_over_tol_where_oracle_within"] == 0, r
    assert r["mismatches_unexplained"] == 0, r


@pytest.mark.parametrize("threads", [1, 8])
def test_fixed_point_sums_vs_f64_sums_planes(oracle_mod, threads):
    pts, w, cfg = _planes()
    it, tol = cfg["iter_count"], cfg["tolerance"]
    a, _ = oracle_mod.rcb(pts, w, it, tol, fsum=oracle_mod.FSUM_FIXED, threads=8)
    b, st = oracle_mod.rcb(pts, w, it, tol, fsum=oracle_mod.FSUM_SEQ, threads=threads, splits=True)
    _assert_criteria(fp.compare(a, b, pts.astype(np.float32), w, it, tol, st["split_pos"]))


@pytest.mark.parametrize("threads", [1, 8])
def test_fixed_point_sums_vs_f64_sums_hexrib(oracle_mod, threads):
    pts, w, cfg = _hex()
    it, tol = cfg["iter_count"], cfg["tolerance"]
    M = oracle_mod.rib_matrix(pts)
    a, _ = oracle_mod.rib(pts, w, it, tol, fsum=oracle_mod.FSUM_FIXED, threads=8, matrix=M)
    b, st = oracle_mod.rib(pts, w, it, tol, fsum=oracle_mod.FSUM_SEQ, threads=threads, matrix=M, splits=True)
    keys = oracle_mod.map_points(pts, M).astype(np.float32)
    _assert_criteria(fp.compare(a, b, keys, w, it, tol, st["split_pos"]))


def _device_run(coupe, pts, w, it, tol, mode, matrix=None):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    d_p = torch.from_numpy(pts).to(dev)
    d_w = torch.from_numpy(w).to(dev)
    d_o = torch.empty(len(pts), dtype=torch.int64, device=dev)
    coupe.rcb_device(d_o, d_p, d_w, it, tol, mode=mode, matrix=matrix)
    st = coupe.last_stats()
    return d_o.cpu().numpy().view(np.uint64), st


@pytest.mark.gpu
@pytest.mark.parametrize("threads", [1, 8])
def test_gpu_vs_reference_f64_sums_planes(coupe, oracle_mod, threads):
    pts, w, cfg = _planes()
    it, tol = cfg["iter_count"], cfg["tolerance"]
    got, st = _device_run(coupe, pts, w, it, tol, "ref32")
    want, ost = oracle_mod.rcb(pts, w, it, tol, fsum=oracle_mod.FSUM_SEQ, threads=threads, splits=True)
    _assert_criteria(fp.compare(got, want, pts.astype(np.float32), w, it, tol, ost["split_pos"]))
    # the total weight against the exact sum and the reference's f64 sum
    exact = math.fsum(w.tolist())
    assert abs(st["root_weight_sum"] - exact) <= st["weight_sum_error_bound"]
    # the quantisation part of the bound is negligible: the total is the
    # exact sum rounded once
    assert st["weight_sum_error_bound"] <= (0.5 + 1e-6) * math.ulp(exact)


@pytest.mark.gpu
def test_gpu_band_vs_reference_f64_sums_planes(coupe, oracle_mod):
    """The band form (decisions of the all-f64 form) against the oracle's f64
    mode with sequential f64 sums: one ulp of an f64 key."""
    pts, w, cfg = _planes()
    it, tol = cfg["iter_count"], cfg["tolerance"]
    got, _ = _device_run(coupe, pts, w, it, tol, "f32key_f64band")
    want, ost = oracle_mod.rcb(pts, w, it, tol, mode=oracle_mod.F64, fsum=oracle_mod.FSUM_SEQ, splits=True)
    _assert_criteria(fp.compare(got, want, pts, w, it, tol, ost["split_pos"], key_dtype=np.float64))


@pytest.mark.gpu
@pytest.mark.parametrize("threads", [1, 8])
def test_gpu_vs_reference_f64_sums_hexrib(coupe, oracle_mod, threads):
    """Rib: the GPU's basis change given to the oracle, so that only the
    weight sums differ."""
    torch = pytest.importorskip("torch")
    pts, w, cfg = _hex()
    it, tol = cfg["iter_count"], cfg["tolerance"]
    M = coupe.rib_matrix_device(torch.from_numpy(pts).to(torch.device("cuda", 0)))
    got, st = _device_run(coupe, pts, w, it, tol, "ref32", matrix=M)
    want, ost = oracle_mod.rib(pts, w, it, tol, fsum=oracle_mod.FSUM_SEQ, threads=threads, matrix=M, splits=True)
    keys = oracle_mod.map_points(pts, M).astype(np.float32)
    _assert_criteria(fp.compare(got, want, keys, w, it, tol, ost["split_pos"]))
    exact = math.fsum(w.tolist())
    assert abs(st["root_weight_sum"] - exact) <= st["weight_sum_error_bound"]
