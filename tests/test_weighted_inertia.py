"""The opt-in weighted inertia of Rib (COUPE_GPU_WEIGHTED_INERTIA; no
counterpart in coupe, whose inertia_matrix is unweighted,
coupe/src/geometry.rs:273-284 — that stays the default and is tested in
tests/test_gpu_parity.py).  Weighted centroid sum(w p) / sum(w) and
M = sum(w (p - c)(p - c)^T), then coupe's eigenvector, Householder
reflection and inverse (geometry.rs:286-319, 219)."""
import numpy as np
import pytest


def _mesh(side, seed, wkind):
    from coupe_gb300 import workloads
    pts, w, _ = workloads.hex_mesh_rib(side=side, seed=seed)
    rng = np.random.default_rng(seed)
    if wkind == "i64":
        w = rng.integers(1, 1000, size=len(pts), dtype=np.int64)
    # a heavy corner pulls the weighted centroid and axes away from the
    # unweighted ones
    w = w.copy()
    heavy = pts[:, 0] > np.quantile(pts[:, 0], 0.9)
    w[heavy] = w[heavy] * 50
    return pts, w


def test_oracle_unit_weights_give_the_unweighted_matrix(oracle_mod):
    pts, _ = _mesh(24, 1, "f64")
    M_u = oracle_mod.rib_matrix(pts)
    M_w = oracle_mod.rib_matrix_weighted(pts, np.ones(len(pts)))
    assert np.allclose(M_u, M_w, rtol=1e-10, atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("wkind", ["i64", "f64"])
@pytest.mark.parametrize("dim", [2, 3])
def test_weighted_matrix_matches_oracle(coupe, oracle_mod, wkind, dim):
    torch = pytest.importorskip("torch")
    pts, w = _mesh(40, 2 + dim, wkind)
    pts = np.ascontiguousarray(pts[:, :dim])
    M_o = oracle_mod.rib_matrix_weighted(pts, w.astype(np.float64))
    M_g = coupe.rib_matrix_device(torch.from_numpy(pts).cuda(), weights=torch.from_numpy(w).cuda())
    assert np.allclose(M_g, M_o, rtol=1e-9, atol=1e-12)
    # and it differs from coupe's unweighted matrix on this input
    assert not np.allclose(M_g, oracle_mod.rib_matrix(pts), rtol=1e-3, atol=1e-6)


@pytest.mark.gpu
def test_unit_weights_give_coupes_matrix(coupe, oracle_mod):
    torch = pytest.importorskip("torch")
    pts, _ = _mesh(40, 9, "f64")
    d = torch.from_numpy(pts).cuda()
    M_w = coupe.rib_matrix_device(d, weights=torch.ones(len(pts), dtype=torch.int64, device="cuda"))
    M_u = coupe.rib_matrix_device(d)
    assert np.allclose(M_w, M_u, rtol=1e-12, atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["ref32", "f32key_f64band"])
def test_weighted_rib_ids(coupe, oracle_mod, mode):
    """Through the C ABI: Rib(weighted_inertia=True) equals the oracle's Rcb
    on the points mapped by the GPU's weighted basis change (bit for bit) and
    nearly all ids of the oracle's own weighted Rib."""
    torch = pytest.importorskip("torch")
    pts, w = _mesh(48, 11, "i64")
    ids = np.zeros(len(pts), dtype=np.uint64)
    coupe.Rib(iter_count=8, tolerance=0.01, mode=mode, weighted_inertia=True).partition(ids, (pts, w))
    M_g = coupe.rib_matrix_device(torch.from_numpy(pts).cuda(), weights=torch.from_numpy(w).cuda())
    omode = oracle_mod.REF32 if mode == "ref32" else oracle_mod.F64
    want, _ = oracle_mod.rib(pts, w, 8, 0.01, mode=omode, matrix=M_g)
    assert (ids == want).all()
    own, _ = oracle_mod.rib(pts, w, 8, 0.01, mode=omode, matrix=oracle_mod.rib_matrix_weighted(pts, w))
    assert (ids == own).mean() >= 0.9999
    # the default is coupe's unweighted Rib
    ids0 = np.zeros(len(pts), dtype=np.uint64)
    coupe.Rib(iter_count=8, tolerance=0.01, mode=mode).partition(ids0, (pts, w))
    assert not (ids0 == ids).all()


@pytest.mark.gpu
def test_weighted_inertia_rejects_zero_weight_sum(coupe):
    torch = pytest.importorskip("torch")
    pts = np.random.default_rng(3).random((1000, 3))
    with pytest.raises(coupe.CoupeError):
        coupe.rib_matrix_device(torch.from_numpy(pts).cuda(), weights=torch.zeros(1000, dtype=torch.float64,
                                                                                 device="cuda"))
