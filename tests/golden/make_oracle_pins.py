"""Generates tests/golden/oracle_pins.json: SHA-256 of the oracle's part ids
(uint64, little endian) on seeded inputs, made on x86_64.  The GPU suite
re-runs the oracle on the GPU host (aarch64) and compares, which pins the
oracle's arithmetic across the two architectures.

Usage: python tests/golden/make_oracle_pins.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

CASES = [
    # name, n, dim, weight kind, iters, tol, mode
    ("uniform2d_i64", 20000, 2, "i64", 6, 0.05, 0),
    ("uniform3d_i32", 20000, 3, "i32", 7, 0.01, 0),
    ("gauss3d_i64_f64keys", 30000, 3, "gauss", 8, 0.01, 1),
    ("uniform3d_f64w_fixed", 20000, 3, "f64", 7, 0.005, 0),
]


def inputs(name, n, dim, wk, seed):
    rng = np.random.default_rng(seed)
    if wk == "gauss":
        from coupe_gb300 import workloads
        pts, w, _ = workloads.gaussian_mixture3d(n=n, seed=seed)
        return pts, w
    pts = rng.random((n, dim))
    if wk == "i64":
        w = rng.integers(1, 100, size=n, dtype=np.int64)
    elif wk == "i32":
        w = rng.integers(1, 100, size=n, dtype=np.int32)
    else:
        w = rng.lognormal(0.0, 1.0, size=n)
    return pts, w


def digest(ids):
    return hashlib.sha256(np.ascontiguousarray(ids, dtype="<u8").tobytes()).hexdigest()


def compute():
    import oracle
    out = {}
    for i, (name, n, dim, wk, iters, tol, mode) in enumerate(CASES):
        pts, w = inputs(name, n, dim, wk, 100 + i)
        ids, _ = oracle.rcb(pts, w, iters, tol, mode=mode)
        out[name] = digest(ids)
    return out


if __name__ == "__main__":
    with open(os.path.join(HERE, "oracle_pins.json"), "w") as f:
        json.dump(compute(), f, indent=1)
    print("wrote", os.path.join(HERE, "oracle_pins.json"))
