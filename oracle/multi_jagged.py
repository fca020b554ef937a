"""TEST INFRASTRUCTURE ONLY — a CPU restatement of coupe's axis_sort and
MultiJagged (coupe/src/algorithms/recursive_bisection.rs:815-827,
coupe/src/algorithms/multi_jagged.rs:75-318), the checker of the GPU's
coupe_gpu_axis_sort_device / coupe_gpu_multi_jagged*.

It follows coupe run by one rayon worker:
  * part ids in the order the recursion meets the leaves (depth first);
  * compute_split_positions' scan with one fold chunk: the total and the
    running weights are sequential f64 sums over the sorted points.
coupe's axis_sort is unstable; this one (a stable sort) keeps equal
coordinates in index order, which is the GPU's order.  Tests use distinct
coordinates where coupe's order matters.
"""
import numpy as np


def compute_modifiers(num_regular_parts, num_fat_parts, num_regular_subparts, num_fat_subparts):
    """multi_jagged.rs:138-149"""
    num_subparts = num_regular_parts * num_regular_subparts + num_fat_parts * num_fat_subparts
    return ([num_fat_subparts / num_subparts] * num_fat_parts
            + [num_regular_subparts / num_subparts] * num_regular_parts)


def partition_scheme(num_parts, max_iter):
    """multi_jagged.rs:75-103, as a dict {num_splits, modifiers, next}.

    The root is (num_parts as f32).powf(1 / max_iter as f32).ceil(); a node
    that does not split is a part, and its children (which coupe builds but
    never visits) are left out.  Raises ValueError where coupe's recursion
    does not end (max_iter exhausted with more than one part left)."""
    with np.errstate(divide="ignore", over="ignore"):
        inv = np.float32(1.0) / np.float32(max_iter)
        root_f = np.ceil(np.power(np.float32(num_parts), inv))
    if not np.isfinite(root_f) or root_f < 1 or root_f >= 2.0 ** 32:
        raise ValueError("no partition scheme for %d parts in %d iterations" % (num_parts, max_iter))
    approx_root = int(root_f)
    rem, quotient = num_parts % approx_root, num_parts // approx_root
    node = {"num_splits": approx_root - 1,
            "modifiers": compute_modifiers(approx_root - rem, rem, quotient, quotient + 1),
            "next": None}
    if node["num_splits"] == 0:
        return node
    if max_iter == 0:
        raise ValueError("no partition scheme for %d parts in 0 iterations" % num_parts)
    node["next"] = [partition_scheme(quotient + 1 if i < rem else quotient, max_iter - 1)
                    for i in range(approx_root)]
    return node


def axis_sort(points, permutation, coord):
    """recursive_bisection.rs:815-827 (stable: ties keep their order)."""
    permutation = np.asarray(permutation, dtype=np.int64)
    return permutation[np.argsort(np.asarray(points)[permutation, coord], kind="stable")]


def _ulps_eq(a, b, max_ulps=4):
    """approx's default f64 ulps comparison (epsilon f64::EPSILON, 4 ulps),
    used at multi_jagged.rs:283-286."""
    if abs(a - b) <= np.finfo(np.float64).eps:
        return True
    if np.signbit(a) != np.signbit(b):
        return False
    x = int(np.float64(a).view(np.int64))
    y = int(np.float64(b).view(np.int64))
    return abs(x - y) <= max_ulps


def compute_split_positions(weights, permutation, modifiers):
    """multi_jagged.rs:222-295 with one scan chunk: for each threshold (the
    running sums of total * modifier over all modifiers but the last) the
    first position whose running weight exceeds it and is not within 4 ulps
    of it.  coupe panics where no such position exists; here the position
    is then len(permutation)."""
    w = [float(weights[i]) for i in permutation]
    total = 0.0
    for x in w:
        total += x
    thresholds, consumed = [], 0.0
    for m in modifiers[:-1]:
        consumed += total * m
        thresholds.append(consumed)
    out, idx, acc = [], 0, 0.0
    for t in thresholds:
        while idx < len(w) and (acc + w[idx] < t or _ulps_eq(t, acc + w[idx])):
            acc += w[idx]
            idx += 1
        out.append(idx)
    return out


def split_at_mut_many(seq, positions):
    """multi_jagged.rs:297-318: the sub-slices between consecutive positions."""
    parts, prev = [], 0
    for p in positions:
        parts.append(seq[prev:p])
        prev = p
    parts.append(seq[prev:])
    return parts


def multi_jagged(points, weights, part_count, max_iter):
    """multi_jagged.rs:150-220: part ids of every point."""
    points = np.asarray(points, dtype=np.float64)
    n, dim = points.shape
    part = np.zeros(n, dtype=np.int64)
    next_id = [0]

    def recurse(perm, coord, scheme):
        if scheme["num_splits"] != 0:
            perm = axis_sort(points, perm, coord)
            pos = compute_split_positions(weights, perm, scheme["modifiers"])
            for sub, child in zip(split_at_mut_many(perm, pos), scheme["next"]):
                recurse(sub, (coord + 1) % dim, child)
        else:
            part[perm] = next_id[0]
            next_id[0] += 1

    recurse(np.arange(n, dtype=np.int64), 0, partition_scheme(part_count, max_iter))
    return part
