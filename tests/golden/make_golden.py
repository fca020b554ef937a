"""Generates tests/golden/reference_known_answers.json.

The inputs are read from the reference's own test sources; the file and line
ranges are recorded next to each case.  The expected answers are the
assertions of those tests, restated as data.  The coupe-ffi rcb.c example
prints its partitions without asserting them; its expected ids are derived by
hand from recursive_bisection.rs:456-705 (iter_count 1 splits x at 0.5;
iter_count 2 then splits y at 0.5 in both halves).

Usage: python tests/golden/make_golden.py /path/to/coupe
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
NUM = r"-?\d+(?:\.\d*)?(?:e-?\d+)?"


def lines(root, rel, a, b):
    with open(os.path.join(root, rel)) as f:
        src = f.read().split("\n")
    return "\n".join(src[a - 1:b])


def points(text):
    pts = []
    for m in re.finditer(r"Point[23]D::(?:new\(([^)]*)\)|from\(\[([^\]]*)\]\))", text):
        body = m.group(1) if m.group(1) is not None else m.group(2)
        pts.append([float(x) for x in re.findall(NUM, body)])
    return pts


def c_points(text):
    return [[float(x) for x in re.findall(NUM, row)] for row in re.findall(r"\{([^{}]*)\}", text)]


def main(root):
    rb = "coupe/src/algorithms/recursive_bisection.rs"
    geo = "coupe/src/geometry.rs"
    cases = {}
    cases["rcb_doctest"] = {
        "source": rb + ":739-768", "points": points(lines(root, rb, 739, 768)),
        "weights": "int32 ones", "iter_count": 2, "tolerance": 0.0,
        "expect": "all ids distinct"}
    cases["rib_doctest"] = {
        "source": rb + ":862-894", "points": points(lines(root, rb, 862, 894)),
        "weights": "int32 ones", "iter_count": 1, "tolerance": 0.0,
        "expect": {"equal": [[0, 1], [2, 3]], "different": [[1, 2]]}}
    cases["test_rcb_basic"] = {
        "source": rb + ":1077-1115", "points": points(lines(root, rb, 1077, 1115)),
        "weights": "f64 ones", "iter_count": 2, "tolerance": 0.05,
        "expect": {"equal": [[0, 6], [1, 7], [2, 5], [3, 4]], "part_sizes": [2, 2, 2, 2]}}
    cases["ffi_example_rcb_c"] = {
        "source": "coupe-ffi/examples/rcb.c:12-36",
        "points": c_points(lines(root, "coupe-ffi/examples/rcb.c", 13, 16)),
        "weights": "int32 constant 1", "tolerance": 0.05,
        "expect": {"iter_count_1": [0, 0, 1, 1], "iter_count_2": [0, 1, 2, 3]}}
    cases["aabb_2d"] = {
        "source": geo + ":341-355", "points": points(lines(root, geo, 341, 355))[:5],
        "expect": {"min": [0.0, 0.0], "max": [5.0, 5.0]}}
    cases["aabb_3d"] = {
        "source": geo + ":489-503", "points": points(lines(root, geo, 489, 503))[:5],
        "expect": {"min": [0.0, 0.0, -2.0], "max": [5.0, 5.0, 5.0]}}
    cases["inertia_matrix"] = {
        "source": geo + ":363-375", "points": points(lines(root, geo, 363, 375)),
        "expect": {"matrix": [[18.0, -18.0], [-18.0, 18.0]]}}
    cases["inertia_vector_2d"] = {
        "source": geo + ":377-393", "points": points(lines(root, geo, 377, 393))[:3],
        "expect": {"parallel_to": [1.0, -1.0], "cross_norm_max": 1e-15}}
    cases["inertia_vector_3d"] = {
        "source": geo + ":505-518", "points": points(lines(root, geo, 505, 518))[:3],
        "expect": {"parallel_to": [1.0, -1.0, -1.0], "cross_norm_max": 1e-15}}
    cases["householder_6d"] = {
        "source": geo + ":460-487", "dim": 6,
        "expect": {"column_norm": 1.0, "orthogonality_eps": 1e-14, "first_column_parallel_eps": 1e-14}}
    cases["par_rcb_split_property"] = {
        "source": rb + ":1041-1075",
        "inputs": "1..200 f32 keys in [0,1), u32 weights 1..999, tolerance 0.05, min/max of the keys",
        "expect": "left < split_pos <= right; weight_left = sum(left); sum - weight_left = sum(right)"}
    cases["reorder_split_scalar_property"] = {
        "source": rb + ":952-983",
        "inputs": "1..23 positive f32 keys, every index as the pivot",
        "expect": "left < pivot <= right; each key on exactly one side"}
    mj = "coupe/src/algorithms/multi_jagged.rs"
    sample = points(lines(root, rb, 940, 950))
    cases["axis_sort_x"] = {
        "source": rb + ":1021-1029", "points": sample, "coord": 0,
        "expect": [int(x) for x in re.findall(r"\d+", lines(root, rb, 1028, 1028).split("vec!")[1])]}
    cases["axis_sort_y"] = {
        "source": rb + ":1031-1039", "points": sample, "coord": 1,
        "expect": [int(x) for x in re.findall(r"\d+", lines(root, rb, 1038, 1038).split("vec!")[1])]}
    cases["multi_jagged_doctest"] = {
        "source": mj + ":333-365", "points": points(lines(root, mj, 338, 348)),
        "weights": "f64 4.2 each", "part_count": 9, "max_iter": 4, "expect": "all ids distinct"}
    cases["split_at_mut_many"] = {
        "source": mj + ":416-433", "len": 13, "positions": [1, 3, 6, 9, 11],
        "expect": [[0], [1, 2], [3, 4, 5], [6, 7, 8], [9, 10], [11, 12]]}
    with open(os.path.join(HERE, "reference_known_answers.json"), "w") as f:
        json.dump(cases, f, indent=1)
    print("wrote", os.path.join(HERE, "reference_known_answers.json"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py /path/to/coupe (the reference's source tree)")
    main(sys.argv[1])
