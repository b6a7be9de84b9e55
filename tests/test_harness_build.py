"""The bench's native driver of the reference's per-signal calling pattern
(libdwt_gb300/harness/calls_1d.c, an OpenMP loop of dwt_cdf97_f_ex_stride_s
calls) builds against the library and exports its entry point; no device
work (the calls themselves run in the GPU bench)."""
import shutil

import pytest


def test_calls_1d_driver_builds():
    if not shutil.which("gcc"):
        pytest.skip("no gcc")
    from libdwt_gb300.buildext import build
    build()
    import bench
    lib = bench.native_calls_1d()
    assert lib is not None, "calls_1d.c did not build"
    assert hasattr(lib, "calls_1d")
