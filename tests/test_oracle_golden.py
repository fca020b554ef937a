"""The oracle against the known answers of coupe's own tests
(tests/golden/reference_known_answers.json, extracted from the reference's
test sources by tests/golden/make_golden.py), and its cross-architecture pin."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
KA = json.load(open(os.path.join(HERE, "golden", "reference_known_answers.json")))


def _w(spec, n):
    if spec.startswith("int32"):
        return np.ones(n, dtype=np.int32)
    return np.ones(n, dtype=np.float64)


def test_rcb_doctest(oracle_mod):
    c = KA["rcb_doctest"]
    ids, _ = oracle_mod.rcb(c["points"], _w(c["weights"], 4), c["iter_count"], c["tolerance"])
    assert len(set(ids.tolist())) == 4


def test_rib_doctest(oracle_mod):
    c = KA["rib_doctest"]
    ids, _ = oracle_mod.rib(c["points"], _w(c["weights"], 4), c["iter_count"], c["tolerance"])
    for a, b in c["expect"]["equal"]:
        assert ids[a] == ids[b]
    for a, b in c["expect"]["different"]:
        assert ids[a] != ids[b]


def test_rcb_basic(oracle_mod):
    c = KA["test_rcb_basic"]
    ids, _ = oracle_mod.rcb(c["points"], _w(c["weights"], 8), c["iter_count"], c["tolerance"])
    for a, b in c["expect"]["equal"]:
        assert ids[a] == ids[b]
    assert sorted(np.bincount(ids.astype(np.int64)).tolist()) == c["expect"]["part_sizes"]


def test_ffi_example(oracle_mod):
    c = KA["ffi_example_rcb_c"]
    w = np.ones(4, dtype=np.int32)
    assert oracle_mod.rcb(c["points"], w, 1, c["tolerance"])[0].tolist() == c["expect"]["iter_count_1"]
    assert oracle_mod.rcb(c["points"], w, 2, c["tolerance"])[0].tolist() == c["expect"]["iter_count_2"]


@pytest.mark.parametrize("name", ["aabb_2d", "aabb_3d"])
def test_bounding_box(oracle_mod, name):
    c = KA[name]
    lo, hi = oracle_mod.bbox(c["points"])
    assert lo.tolist() == c["expect"]["min"] and hi.tolist() == c["expect"]["max"]


def test_inertia_matrix(oracle_mod):
    c = KA["inertia_matrix"]
    assert oracle_mod.inertia_matrix(c["points"]).tolist() == c["expect"]["matrix"]


@pytest.mark.parametrize("name", ["inertia_vector_2d", "inertia_vector_3d"])
def test_inertia_vector(oracle_mod, name):
    c = KA[name]
    v = oracle_mod.inertia_vector(oracle_mod.inertia_matrix(c["points"]))
    e = np.array(c["expect"]["parallel_to"], dtype=float)
    v3, e3 = np.zeros(3), np.zeros(3)
    v3[:len(v)], e3[:len(e)] = v, e
    assert np.linalg.norm(np.cross(e3, v3)) <= c["expect"]["cross_norm_max"]


def test_householder_6d(oracle_mod):
    c = KA["householder_6d"]
    rng = np.random.default_rng(7)
    for _ in range(20):
        el = rng.random(c["dim"])
        h = oracle_mod.householder(el)
        for col in range(c["dim"]):
            assert abs(np.linalg.norm(h[:, col]) - 1.0) <= 4 * np.finfo(float).eps
        g = h.T @ h
        off = g - np.diag(np.diag(g))
        assert np.abs(off).max() <= c["expect"]["orthogonality_eps"]
        u = el / np.linalg.norm(el)
        assert np.abs(u * (u @ h[:, 0]) - h[:, 0]).max() <= c["expect"]["first_column_parallel_eps"]


def test_par_rcb_split_property(oracle_mod):
    """recursive_bisection.rs:1041-1075 on 300 seeded cases."""
    rng = np.random.default_rng(11)
    for _ in range(300):
        n = int(rng.integers(1, 200))
        keys = rng.random(n).astype(np.float32)
        w = rng.integers(1, 1000, size=n).astype(np.uint32)
        L, R, wl_, wr_, wl, sp = oracle_mod.split_f32_u32(keys, w, 0.05, keys.min(), keys.max())
        assert (L < np.float32(sp)).all() and (np.float32(sp) <= R).all()
        assert wl == int(wl_.sum())
        assert (int(w.sum()) - wl) == int(wr_.sum())


def test_reorder_split_scalar_property(oracle_mod):
    """recursive_bisection.rs:952-983 on seeded cases, every pivot."""
    rng = np.random.default_rng(12)
    for _ in range(200):
        n = int(rng.integers(1, 24))
        keys = (rng.random(n) * 1e3).astype(np.float32) + np.float32(1e-3)
        for p in range(n):
            L, R = oracle_mod.reorder_split_f32(keys, p)
            assert (L < keys[p]).all() and (keys[p] <= R).all()
            assert sorted(np.concatenate([L, R]).tolist()) == sorted(keys.tolist())


def test_fixed_point_sum_is_order_independent(oracle_mod):
    rng = np.random.default_rng(13)
    w = rng.lognormal(0.0, 2.0, size=10000) * np.where(rng.random(10000) < 0.3, -1, 1)
    s = oracle_mod.fixed_scale(w)
    a = oracle_mod.fixed_sum(w, s)
    b = oracle_mod.fixed_sum(w[::-1].copy(), s)
    c = oracle_mod.fixed_sum(rng.permutation(w), s)
    assert a == b == c
    assert abs(a - np.sum(w.astype(np.longdouble))) <= 1e-12 * np.abs(w).sum()


@pytest.mark.gpu
def test_oracle_pins_across_architectures():
    """Runs with the GPU suite so that it executes on the GPU host (aarch64):
    the oracle gives the ids it gave on x86_64."""
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_oracle_pins
    want = json.load(open(os.path.join(HERE, "golden", "oracle_pins.json")))
    assert make_oracle_pins.compute() == want
