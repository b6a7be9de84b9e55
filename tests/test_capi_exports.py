"""The C-ABI library builds for sm_103a, loads, and exports every symbol that
include/libdwt.h declares.  No GPU work is done here."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "libdwt.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"DWT_EXPORT[^;(]*?\b(dwt_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from libdwt_gb300.buildext import build
    path = build()
    return ctypes.CDLL(path), path


def test_header_declares_the_hot_path():
    syms = declared_symbols()
    for name in ("dwt_cdf97_2f_s", "dwt_cdf97_2i_s", "dwt_cdf53_2f_s", "dwt_cdf53_2i_s",
                 "dwt_cdf97_f_ex_stride_s", "dwt_cdf97_i_ex_stride_s", "dwt_util_init",
                 "dwt_util_finish"):
        assert name in syms


def test_every_declared_symbol_is_exported(lib):
    L, path = lib
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    for s in declared_symbols():
        getattr(L, s)


def test_host_helpers(lib):
    L, _ = lib
    L.dwt_util_ceil_log2.argtypes = [ctypes.c_int]
    L.dwt_util_pow2_ceil_log2.argtypes = [ctypes.c_int]
    for x, e in [(1, 0), (2, 1), (3, 2), (4, 2), (5, 3), (1024, 10), (1025, 11), (16383, 14)]:
        assert L.dwt_util_ceil_log2(x) == e
        assert L.dwt_util_pow2_ceil_log2(x) == 1 << e
    L.dwt_gpu_error_string.restype = ctypes.c_char_p
    assert L.dwt_gpu_error_string(-1) == b"invalid argument"


def test_dense_launch_plan(lib):
    """One level kernel per level down to the coarse kernel's band (at most
    64 x 64 pixels), then one coarse launch: the count bench.py reports."""
    L, _ = lib
    L.dwt_gpu_dense_launches.argtypes = [ctypes.c_int] * 3
    assert L.dwt_gpu_dense_launches(16384, 16384, 14) == 9   # 16384^2 .. 128^2, then 64^2 .. 1
    assert L.dwt_gpu_dense_launches(16384, 16384, -1) == 9
    assert L.dwt_gpu_dense_launches(16383, 16385, 14) == 10  # its 64 x 65 band is above 4096 pixels
    assert L.dwt_gpu_dense_launches(1024, 1024, 5) == 5
    assert L.dwt_gpu_dense_launches(64, 64, 6) == 1
    assert L.dwt_gpu_dense_launches(128, 128, 1) == 1        # one level, no coarse launch
    assert L.dwt_gpu_dense_launches(8, 8, 0) == 0
    assert L.dwt_gpu_dense_launches(0, 8, 1) == -1
