"""Failure detection without faulting the GPU: every device-side wait of the
kernels is bounded and reports through an error word.  A one-warp kernel
waits on an mbarrier that nothing completes, with a short limit; the call
must return DWT_GPU_EDEVICE, log the code, clear the word, and leave the
context usable (the next transform is bit-exact)."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module")
def L():
    from libdwt_gb300.buildext import build
    lib = C.CDLL(build())
    lib.dwt_gpu_selftest_wait_timeout.argtypes = [C.c_int]
    return lib


def test_invalid_limit_is_refused_before_any_device_work(L):
    assert L.dwt_gpu_selftest_wait_timeout(0) == -1
    assert L.dwt_gpu_selftest_wait_timeout(-5) == -1


@pytest.mark.gpu
def test_wait_that_runs_out_reports_and_the_context_survives(L, capfd):
    import libdwt_gb300 as D
    rc = L.dwt_gpu_selftest_wait_timeout(2000)
    err = capfd.readouterr().err
    assert rc == -4  # DWT_GPU_EDEVICE
    assert "device-side wait gave up (code 1)" in err
    assert L.dwt_gpu_get_last_error() == -4
    # the error word was cleared and the context still works
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, size=(300, 257)).astype(np.float32)
    ref, j = O.transform2_dense(img, "cdf97", "f", -1)
    buf = img.copy()
    assert D.transform2(buf, "cdf97", "f", 257 * 4, 4, (257, 300), (257, 300), -1) == j
    assert np.array_equal(buf, ref)
    assert L.dwt_gpu_get_last_error() == 0
    assert L.dwt_gpu_sync_check() == 0


def test_inplace_wait_invalid_limit_is_refused(L):
    L.dwt_gpu_selftest_inplace_wait_timeout.argtypes = [C.c_int]
    assert L.dwt_gpu_selftest_inplace_wait_timeout(0) == -1


@pytest.mark.gpu
def test_inplace_order_wait_that_runs_out_reports(L, capfd):
    """The wait of an ordered in-place unit for earlier segments that never
    finish gives up, raises its code (2) and leaves the context usable."""
    import libdwt_gb300 as D
    L.dwt_gpu_selftest_inplace_wait_timeout.argtypes = [C.c_int]
    rc = L.dwt_gpu_selftest_inplace_wait_timeout(2000)
    err = capfd.readouterr().err
    assert rc == -4  # DWT_GPU_EDEVICE
    assert "device-side wait gave up (code 2)" in err
    rng = np.random.default_rng(4)
    img = rng.integers(0, 256, size=(260, 301)).astype(np.float32)
    ref, j = O.transform2_dense(img, "cdf53", "f", -1)
    buf = img.copy()
    assert D.transform2(buf, "cdf53", "f", 301 * 4, 4, (301, 260), (301, 260), -1) == j
    assert np.array_equal(buf, ref)
