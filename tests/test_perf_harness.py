"""libdwt's performance harness and its host utilities, exported by this
library (src/libdwt.c:1051-1277, 6834-7120, 8386-9036).  Host-only checks run
on the CPU; the harness itself drives the GPU path and is marked gpu."""
import ctypes as C
import math
import os

import numpy as np
import pytest


@pytest.fixture(scope="module")
def L():
    import libdwt_gb300 as D
    L = D.lib()
    vp, i = C.c_void_p, C.c_int
    L.dwt_util_test_image_fill_s.argtypes = [vp, i, i, i, i, i]
    L.dwt_util_test_image_fill_s.restype = None
    L.dwt_util_test_image_fill_d.argtypes = [vp, i, i, i, i, i]
    L.dwt_util_test_image_fill_d.restype = None
    L.dwt_util_compare_s.argtypes = [vp, vp, i, i, i, i]
    L.dwt_util_compare_d.argtypes = [vp, vp, i, i, i, i]
    L.dwt_util_get_clock.restype = C.c_int64
    L.dwt_util_get_frequency.restype = C.c_int64
    L.dwt_util_perf_cdf97_2_s.argtypes = [i] * 12 + [C.POINTER(C.c_float)] * 2
    L.dwt_util_perf_cdf97_2_s.restype = None
    L.dwt_util_measure_perf_cdf97_2_s.argtypes = [i] * 10 + [vp, vp]
    L.dwt_util_measure_perf_cdf97_2_s.restype = None
    return L


def test_test_image_matches_reference(L, golden):
    # the golden example_simple case starts from the reference's own pattern
    c = golden.cases("example_simple")[0]
    inp, _ = golden.io(c)
    img = np.zeros((c["oy"], c["ox"]), np.float32)
    L.dwt_util_test_image_fill_s(img.ctypes.data, c["ox"] * 4, 4, c["ox"], c["oy"], 0)
    assert np.array_equal(img.view(np.uint32), inp.reshape(img.shape).view(np.uint32))
    # the double pattern is the same formula in double
    d = np.zeros((5, 7), np.float64)
    L.dwt_util_test_image_fill_d(d.ctypes.data, 7 * 8, 8, 7, 5, 1)
    want = [[2 * (x >> 1) * y / float((x >> 1) ** 2 + y * y + 1) for x in range(7)] for y in range(5)]
    assert np.array_equal(d, np.array(want))


def test_compare(L):
    a = np.arange(12, dtype=np.float32).reshape(3, 4)
    b = a.copy()
    assert L.dwt_util_compare_s(a.ctypes.data, b.ctypes.data, 16, 4, 4, 3) == 0
    b[1, 2] += 2e-3
    assert L.dwt_util_compare_s(a.ctypes.data, b.ctypes.data, 16, 4, 4, 3) == 1
    b[1, 2] = a[1, 2] + 5e-4
    assert L.dwt_util_compare_s(a.ctypes.data, b.ctypes.data, 16, 4, 4, 3) == 0
    b[0, 0] = np.nan
    assert L.dwt_util_compare_s(a.ctypes.data, b.ctypes.data, 16, 4, 4, 3) == 1
    x = np.ones((2, 2)), np.ones((2, 2)) + 2e-6
    assert L.dwt_util_compare_d(x[0].ctypes.data, x[1].ctypes.data, 16, 8, 2, 2) == 1


def test_clocks(L):
    t = L.dwt_util_clock_autoselect()
    assert t == 0  # DWT_TIME_CLOCK_GETTIME, as the reference with clock_gettime available
    for typ in (t, 2, 6, 12, 14):
        f = L.dwt_util_get_frequency(typ)
        assert f > 0
        a = L.dwt_util_get_clock(typ)
        b = L.dwt_util_get_clock(typ)
        assert b >= a
    assert L.dwt_util_get_max_threads() == 1


@pytest.mark.gpu
def test_perf_and_measure(L, tmp_path):
    fs, is_ = C.c_float(), C.c_float()
    L.dwt_util_perf_cdf97_2_s(256 * 4, 4, 256, 256, 256, 256, -1, 0, 0, 2, 3, 0, C.byref(fs), C.byref(is_))
    assert 0 < fs.value < 1 and 0 < is_.value < 1
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    ff = libc.fopen(str(tmp_path / "fwd.txt").encode(), b"w")
    fi = libc.fopen(str(tmp_path / "inv.txt").encode(), b"w")
    # DWT_ARR_PACKED, 1..300, no optimal stride, full depth, decompose to one
    L.dwt_util_measure_perf_cdf97_2_s(2, 1, 300, 0, -1, 1, 0, 1, 2, 0, ff, fi)
    libc.fclose(ff)
    libc.fclose(fi)
    sizes, x = [], 1
    while x <= 300:
        sizes.append(x * x)
        x = int(math.ceil(np.float32(x) * np.float32(1.28)))
    for name in ("fwd.txt", "inv.txt"):
        lines = (tmp_path / name).read_text().splitlines()
        assert [int(l.split("\t")[0]) for l in lines] == sizes
        assert all(len(l.split("\t")[1].split(".")[1]) == 10 and float(l.split("\t")[1]) > 0 for l in lines)
