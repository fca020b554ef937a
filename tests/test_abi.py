"""CPU checks of the C ABI: the library loads without a GPU, exports every
symbol the headers declare, and validates arguments like coupe-ffi before
touching the device (coupe-ffi/src/lib.rs:272-304)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for h in ("coupe.h", "coupe_gpu.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"\b(coupe_\w+)\s*\(", src)
    return sorted(set(names))


def test_exports_every_declared_symbol(coupe):
    L = coupe.lib()
    declared = _declared()
    assert "coupe_rcb" in declared and "coupe_rib" in declared
    for name in declared:
        assert hasattr(L, name), name
    assert sorted(declared) == sorted(coupe.EXPORTED)


def test_strerror_matches_reference_messages(coupe):
    L = coupe.lib()
    # coupe-ffi/src/lib.rs:69-110
    assert L.coupe_strerror(0) == b"success"
    assert L.coupe_strerror(1) == b"allocation failed"
    assert L.coupe_strerror(3) == b"this algorithm does not support the given mesh dimension"
    assert L.coupe_strerror(6) == b"input iters (e.g. weights and points) don't have the same length"


def _data(L, coupe, arr, t):
    return L.coupe_data_array(len(arr), t, arr.ctypes.data)


def test_len_mismatch_before_bad_dimension(coupe):
    """A length mismatch is reported first, even with a bad dimension."""
    L = coupe.lib()
    pts = np.zeros((4, 2))
    w = np.ones(3, dtype=np.int64)
    dp, dw = _data(L, coupe, pts, coupe.COUPE_DOUBLE), _data(L, coupe, w, coupe.COUPE_INT64)
    part = np.zeros(4, dtype=np.uint64)
    assert L.coupe_rcb(part.ctypes.data, 7, dp, dw, 2, 0.05) == coupe.ERR_LEN_MISMATCH
    assert L.coupe_rib(part.ctypes.data, 2, dp, dw, 2, 0.05) == coupe.ERR_LEN_MISMATCH
    L.coupe_data_free(dp)
    L.coupe_data_free(dw)


def test_bad_dimension(coupe):
    L = coupe.lib()
    pts = np.zeros((4, 2))
    w = np.ones(4, dtype=np.int64)
    dp, dw = _data(L, coupe, pts, coupe.COUPE_DOUBLE), _data(L, coupe, w, coupe.COUPE_INT64)
    part = np.zeros(4, dtype=np.uint64)
    for d in (0, 1, 4, 5):
        assert L.coupe_rcb(part.ctypes.data, d, dp, dw, 2, 0.05) == coupe.ERR_BAD_DIMENSION
        assert L.coupe_rib(part.ctypes.data, d, dp, dw, 2, 0.05) == coupe.ERR_BAD_DIMENSION
    L.coupe_data_free(dp)
    L.coupe_data_free(dw)


def test_empty_input_is_ok_and_untouched(coupe):
    """rcb returns Ok(()) on empty input (recursive_bisection.rs:685-688)."""
    L = coupe.lib()
    pts = np.zeros((0, 3))
    w = np.zeros(0, dtype=np.int64)
    dp, dw = _data(L, coupe, pts, coupe.COUPE_DOUBLE), _data(L, coupe, w, coupe.COUPE_INT64)
    sentinel = np.array([7], dtype=np.uint64)
    assert L.coupe_rcb(sentinel.ctypes.data, 3, dp, dw, 5, 0.05) == coupe.ERR_OK
    assert sentinel[0] == 7
    L.coupe_data_free(dp)
    L.coupe_data_free(dw)


def test_data_free_null_is_noop(coupe):
    coupe.lib().coupe_data_free(None)


def test_version(coupe):
    assert b"sm_103a" in coupe.lib().coupe_gpu_version()


def test_batched_arguments_checked_before_the_device(coupe):
    """coupe_gpu_rcb_batched validates its host arrays before any device
    work: the device pointers below are never dereferenced."""
    L = coupe.lib()
    f = L.coupe_gpu_rcb_batched
    it = np.array([3, 3], dtype=np.uint32)
    bad_start = np.array([1, 5, 9], dtype=np.uint64)
    decreasing = np.array([0, 5, 4], dtype=np.uint64)
    empty = np.array([0, 0, 0], dtype=np.uint64)
    dev = 256  # placeholder device addresses, never used
    assert f(dev, 2, bad_start.ctypes.data, 2, dev, coupe.COUPE_INT64, dev, it.ctypes.data, 0.1, 0, None) == \
        coupe.ERR_LEN_MISMATCH
    assert f(dev, 2, decreasing.ctypes.data, 2, dev, coupe.COUPE_INT64, dev, it.ctypes.data, 0.1, 0, None) == \
        coupe.ERR_LEN_MISMATCH
    assert f(dev, 2, empty.ctypes.data, 4, dev, coupe.COUPE_INT64, dev, it.ctypes.data, 0.1, 0, None) == \
        coupe.ERR_BAD_DIMENSION
    assert f(dev, 2, empty.ctypes.data, 3, dev, 7, dev, it.ctypes.data, 0.1, 0, None) == coupe.ERR_BAD_TYPE
    assert f(dev, 0, None, 3, dev, coupe.COUPE_INT64, dev, None, 0.1, 0, None) == coupe.ERR_OK
    assert f(dev, 2, empty.ctypes.data, 3, dev, coupe.COUPE_INT64, dev, it.ctypes.data, 0.1, 0, None) == coupe.ERR_OK
    assert f(dev, 2, None, 3, dev, coupe.COUPE_INT64, dev, None, 0.1, 0, None) == coupe.ERR_LEN_MISMATCH


def test_headers_compile_as_c_and_cpp(tmp_path):
    """include/*.h are plain C headers (a C or C++ program can bind them)."""
    import shutil
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "h.c"
    src.write_text('#include "coupe.h"\n#include "coupe_gpu.h"\nint main(void) { return 0; }\n')
    for cc, args in (("gcc", ["-std=c99", "-pedantic"]), ("g++", ["-std=c++17", "-x", "c++"])):
        if shutil.which(cc) is None:
            continue
        r = subprocess.run([cc, "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", os.path.join(root, "include")]
                           + args + [str(src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_python_argument_checks_before_the_device(coupe):
    """Length checks of the Python mirror raise before any device work."""
    with pytest.raises(coupe.CoupeError):
        coupe.compute_parts_load(np.array([0, 1], dtype=np.uint64), 2, np.array([1]))
    with pytest.raises(coupe.CoupeError):
        coupe.imbalance(2, np.array([0, 1], dtype=np.uint64), np.array([1, 2, 3]))
    with pytest.raises(coupe.CoupeError):
        coupe.Grid(3, 4).rcb(np.zeros(11, dtype=np.uint64), np.ones(12), 2, threads=4)
    with pytest.raises(coupe.CoupeError):
        coupe.Grid(3, 4).rcb(np.zeros(12, dtype=np.uint64), np.ones(12), 2, threads=1)
