"""TEST INFRASTRUCTURE ONLY — float-weight parity criteria (the checker of
tests/test_float_parity.py and of bench.py's f64-weight workloads).

With f64 weights coupe's sums depend on the summation order (rayon's fold
and reduce, coupe/src/algorithms/recursive_bisection.rs:478-520, 684), while
the GPU sums an order-independent 128-bit fixed point.  Two partitions of the
same points are then compared by the three criteria the GPU form promises:

  1. the share of identical part ids (at least 99.99 %);
  2. per split (tree node): the achieved imbalance |W_left - W/2| / (W/2),
     from exact-ish f64 sums of the final parts, is within the tolerance
     wherever the other partition's is (or no worse than it);
  3. every point whose ids differ is accounted for by split positions within
     one ulp: at the first tree node where the two partitions send it to
     different children, its key lies within one ulp (of the key type) of
     the other partition's split position there.
"""
import numpy as np


def _node_sums(heap, w, iters):
    """Weight and count of every tree node (heap numbering) from leaf heap ids."""
    base = (1 << iters) - 1
    nn = (1 << (iters + 1)) - 1
    W = np.zeros(nn)
    C = np.zeros(nn, dtype=np.int64)
    W[base:] = np.bincount(heap - base, weights=w, minlength=1 << iters)
    C[base:] = np.bincount(heap - base, minlength=1 << iters)
    for d in range(iters - 1, -1, -1):
        lo, hi = (1 << d) - 1, (1 << (d + 1)) - 1
        idx = np.arange(lo, hi)
        W[idx] = W[2 * idx + 1] + W[2 * idx + 2]
        C[idx] = C[2 * idx + 1] + C[2 * idx + 2]
    return W, C


def _imbalance(W, C, iters):
    n_int = (1 << iters) - 1
    idx = np.arange(n_int)
    half = W[idx] / 2.0
    with np.errstate(divide="ignore", invalid="ignore"):
        imb = np.abs(W[2 * idx + 1] - half) / half
    imb[C[idx] < 2] = 0.0  # nothing to balance
    return imb


def compare(ids_a, ids_b, keys, w, iters, tol, split_pos_b, key_dtype=np.float32):
    """Criteria of partition a (the GPU's) against b (the oracle's).

    keys: (n, dim) array of the keys the bisection compared (the f32 keys of
    the REF32 form, after Rib's basis change for Rib); split_pos_b: the
    oracle's split position per heap id.  Returns a dict of figures."""
    ids_a = np.asarray(ids_a, dtype=np.int64)
    ids_b = np.asarray(ids_b, dtype=np.int64)
    n, dim = keys.shape
    base = (1 << iters) - 1
    assert ids_a.max() < (1 << iters) and ids_b.max() < (1 << iters)
    ha, hb = ids_a + base, ids_b + base
    same = ha == hb
    out = {"points": int(n), "identical": float(same.mean()), "mismatches": int((~same).sum())}
    # 2. per-split achieved imbalance
    Wa, Ca = _node_sums(ha, w, iters)
    Wb, Cb = _node_sums(hb, w, iters)
    ia, ib = _imbalance(Wa, Ca, iters), _imbalance(Wb, Cb, iters)
    eps = 1e-9
    real = (Ca[:base] >= 2) | (Cb[:base] >= 2)  # nodes split in either partition
    ok_b = (ib <= tol) & real
    out["splits"] = int(real.sum())
    out["splits_within_tol_oracle"] = int(ok_b.sum())
    out["splits_within_tol_gpu"] = int(((ia <= tol) & real).sum())
    out["splits_over_tol_where_oracle_within"] = int((ok_b & (ia > tol + eps) & (ia > ib + eps)).sum())
    out["max_imbalance_gpu"] = float(np.nanmax(ia)) if base else 0.0
    out["max_imbalance_oracle"] = float(np.nanmax(ib)) if base else 0.0
    # 3. mismatches traced to the first diverging node
    bad = np.nonzero(~same)[0]
    ga, gb = ha[bad].copy(), hb[bad].copy()
    for _ in range(iters):
        m = ga != gb
        if not m.any():
            break
        ga[m] = (ga[m] - 1) // 2
        gb[m] = (gb[m] - 1) // 2
    node = ga
    depth = np.floor(np.log2(node + 1)).astype(np.int64)
    axis = depth % dim
    k = keys[bad, axis].astype(key_dtype)
    t = split_pos_b[node].astype(key_dtype)
    ulp = np.spacing(np.abs(t)).astype(np.float64)
    dist = np.abs(k.astype(np.float64) - t.astype(np.float64))
    within = np.isfinite(t) & (dist <= ulp)
    out["mismatches_within_one_ulp"] = int(within.sum())
    out["mismatches_unexplained"] = int((~within).sum())
    out["mismatch_nodes"] = sorted(set(int(x) for x in np.unique(node)))[:20]
    return out
