"""dwt_gpu_2_dev_noalloc, the entry point for callers that may not allocate
device memory (its scratch is a fixed array inside the library): called
through the C ABI, its output must equal the regular dwt_gpu_2_dev's bit for
bit, on two calls in a row (the array keeps the first call's contents), and
an image too large for the array must be refused without running.

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test."""
import ctypes as C
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    import libdwt_gb300 as D
    L = D.lib()
    f = L.dwt_gpu_2_dev_noalloc
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong, C.c_int,
                  C.c_int, C.c_int, C.c_int, C.c_void_p]
    f.restype = C.c_int
    L.dwt_gpu_selftest_noalloc_wait_timeout.argtypes = [C.c_int]
    L.dwt_gpu_selftest_noalloc_wait_timeout.restype = C.c_int
    L.dwt_gpu_sync_check.restype = C.c_int
    return D, L, torch


def _run(fn, wav, inv, src, dst, j):
    h, w = dst.shape
    return fn(wav, inv, src.data_ptr(), src.stride(0) * 4, dst.data_ptr(), dst.stride(0) * 4, w, h, j, 0,
              None)


def test_noalloc_matches_pooled_path_two_calls(env):
    D, L, torch = env
    rng = np.random.default_rng(99)
    cases = [(2048, 2048, "cdf97"), (1023, 777, "cdf53")]
    for (w, h, wav_name) in cases:
        wav = D.CDF97 if wav_name == "cdf97" else D.CDF53
        pw = (w + 3) // 4 * 4
        img = rng.integers(0, 256, size=(h, w)).astype(np.float32)
        src = torch.zeros((h, pw), dtype=torch.float32, device="cuda")
        src[:, :w] = torch.from_numpy(img).cuda()
        ref = torch.empty((h, w), dtype=torch.float32, device="cuda")
        got = torch.full((h, w), float("nan"), dtype=torch.float32, device="cuda")
        j_ref = _run(L.dwt_gpu_2_dev, wav, 0, src[:, :w], ref, -1)
        j_got = _run(L.dwt_gpu_2_dev_noalloc, wav, 0, src[:, :w], got, -1)
        torch.cuda.synchronize()
        assert j_ref == j_got > 0
        assert torch.equal(got, ref), f"{w}x{h} {wav_name} forward differs"
        # inverse of those coefficients, both ways
        src[:, :w] = ref
        back_ref = torch.empty_like(ref)
        back_got = torch.full_like(ref, float("nan"))
        _run(L.dwt_gpu_2_dev, wav, 1, src[:, :w], back_ref, j_ref)
        assert _run(L.dwt_gpu_2_dev_noalloc, wav, 1, src[:, :w], back_got, j_ref) == j_ref
        torch.cuda.synchronize()
        assert torch.equal(back_got, back_ref), f"{w}x{h} {wav_name} inverse differs"


def test_noalloc_refuses_oversize(env):
    D, L, torch = env
    w = h = 4096
    src = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    dst = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    rc = _run(L.dwt_gpu_2_dev_noalloc, D.CDF97, 0, src, dst, -1)
    torch.cuda.synchronize()
    assert rc == -1  # DWT_GPU_EINVAL
    assert int(torch.count_nonzero(dst)) == 0


def _pair(torch, rng, w, h, pw=None):
    pw = pw or (w + 3) // 4 * 4
    img = rng.integers(0, 256, size=(h, w)).astype(np.float32)
    src = torch.zeros((h, pw), dtype=torch.float32, device="cuda")
    src[:, :w] = torch.from_numpy(img).cuda()
    return src


def test_noalloc_at_the_size_limit_and_on_a_side_stream(env):
    """4095 x 1024 with decompose_one (12 levels) needs exactly the scratch
    of 2048 x 2048, just under the array's size; 2048 x 2049 needs more and is
    refused.  Both directions, on a non-default stream, equal to the pooled
    path bit for bit."""
    D, L, torch = env
    rng = np.random.default_rng(5)
    w, h = 4095, 1024
    src = _pair(torch, rng, w, h)
    side = torch.cuda.Stream()
    for wav in (D.CDF97, D.CDF53):
        ref = torch.empty((h, w), dtype=torch.float32, device="cuda")
        got = torch.full((h, w), float("nan"), dtype=torch.float32, device="cuda")
        jr = L.dwt_gpu_2_dev(wav, 0, src.data_ptr(), src.stride(0) * 4, ref.data_ptr(), w * 4, w, h, -1, 1, None)
        torch.cuda.synchronize()
        jg = L.dwt_gpu_2_dev_noalloc(wav, 0, src.data_ptr(), src.stride(0) * 4, got.data_ptr(), w * 4, w, h, -1,
                                     1, C.c_void_p(side.cuda_stream))
        side.synchronize()
        assert jr == jg == 12
        assert torch.equal(got, ref)
        back_ref = torch.empty_like(ref)
        back_got = torch.full_like(ref, float("nan"))
        cref = torch.zeros_like(src)
        cref[:, :w] = ref
        L.dwt_gpu_2_dev(wav, 1, cref.data_ptr(), cref.stride(0) * 4, back_ref.data_ptr(), w * 4, w, h, 12, 1, None)
        torch.cuda.synchronize()
        assert L.dwt_gpu_2_dev_noalloc(wav, 1, cref.data_ptr(), cref.stride(0) * 4, back_got.data_ptr(), w * 4,
                                       w, h, 12, 1, C.c_void_p(side.cuda_stream)) == 12
        side.synchronize()
        assert torch.equal(back_got, back_ref)
    big = _pair(torch, rng, 2048, 2049)
    out = torch.zeros((2049, 2048), dtype=torch.float32, device="cuda")
    assert L.dwt_gpu_2_dev_noalloc(D.CDF97, 0, big.data_ptr(), big.stride(0) * 4, out.data_ptr(), 2048 * 4, 2048,
                                   2049, -1, 0, None) == -1
    torch.cuda.synchronize()
    assert int(torch.count_nonzero(out)) == 0


def test_overlapping_frames_refused(env):
    """Both device forms work out of place: a destination that overlaps the
    source (in place, or shifted by a row) is refused before anything runs."""
    D, L, torch = env
    rng = np.random.default_rng(6)
    w, h = 256, 128
    buf = _pair(torch, rng, w, h + 1)
    before = buf.clone()
    p, pitch = buf.data_ptr(), buf.stride(0) * 4
    for fn in (L.dwt_gpu_2_dev, L.dwt_gpu_2_dev_noalloc):
        for dst in (p, p + pitch, p + 4):
            assert fn(D.CDF97, 0, p, pitch, dst, pitch, w, h, -1, 0, None) == -1
    torch.cuda.synchronize()
    assert torch.equal(buf, before)
    # zero levels is a copy, and in place it is nothing at all
    assert L.dwt_gpu_2_dev_noalloc(D.CDF97, 0, p, pitch, p, pitch, w, h, 0, 0, None) == 0


def test_noalloc_device_wait_timeout_is_reported(env):
    """A bounded device-side wait that gives up on this path sets its error
    word; dwt_gpu_sync_check reports it once (DWT_GPU_EDEVICE) and clears it,
    and the next call is bit-exact again.  No fault: the wait is the level
    kernels' own bounded mbarrier wait, on a barrier nothing completes."""
    D, L, torch = env
    torch.cuda.synchronize()
    assert L.dwt_gpu_sync_check() == 0
    assert L.dwt_gpu_selftest_noalloc_wait_timeout(0) == -1
    assert L.dwt_gpu_selftest_noalloc_wait_timeout(2000) == 0
    assert L.dwt_gpu_sync_check() == -4  # DWT_GPU_EDEVICE
    assert L.dwt_gpu_sync_check() == 0
    rng = np.random.default_rng(7)
    w, h = 333, 517
    src = _pair(torch, rng, w, h)
    ref = torch.empty((h, w), dtype=torch.float32, device="cuda")
    got = torch.full((h, w), float("nan"), dtype=torch.float32, device="cuda")
    L.dwt_gpu_2_dev(D.CDF97, 0, src.data_ptr(), src.stride(0) * 4, ref.data_ptr(), w * 4, w, h, -1, 0, None)
    L.dwt_gpu_2_dev_noalloc(D.CDF97, 0, src.data_ptr(), src.stride(0) * 4, got.data_ptr(), w * 4, w, h, -1, 0,
                            None)
    assert L.dwt_gpu_sync_check() == 0
    assert torch.equal(got, ref)


_FRESH = textwrap.dedent("""
    import ctypes as C, sys
    import numpy as np, torch
    sys.path.insert(0, {root!r})
    import libdwt_gb300 as D
    L = D.lib()
    f = L.dwt_gpu_2_dev_noalloc
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong, C.c_int,
                  C.c_int, C.c_int, C.c_int, C.c_void_p]
    L.dwt_gpu_sync_check.restype = C.c_int
    rng = np.random.default_rng(8)
    src = torch.from_numpy(rng.integers(0, 256, size=(2048, 2048)).astype(np.float32)).cuda()
    dst = torch.empty_like(src)
    back = torch.empty_like(src)
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    # small calls first load the library's device code (every kernel the
    # measured calls use, and the module holding the fixed array); from then
    # on nothing may change the free device memory
    for wav in (D.CDF97, D.CDF53):
        j = f(wav, 0, src.data_ptr(), 8192, dst.data_ptr(), 8192, 300, 300, -1, 0, None)
        assert j == 9
        assert f(wav, 1, dst.data_ptr(), 8192, back.data_ptr(), 8192, 300, 300, j, 0, None) == j
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for (w, h, wav) in ((2048, 2048, D.CDF97), (1500, 999, D.CDF53), (2047, 1023, D.CDF97)):
        j = f(wav, 0, src.data_ptr(), 8192, dst.data_ptr(), 8192, w, h, -1, 0, None)
        assert j > 0
        # calls share the fixed array: the next one may start only when this
        # one is done (the two streams are not ordered otherwise)
        torch.cuda.synchronize()
        assert f(wav, 1, dst.data_ptr(), 8192, back.data_ptr(), 8192, w, h, j, 0,
                 C.c_void_p(side.cuda_stream)) == j
        side.synchronize()
    assert L.dwt_gpu_sync_check() == 0
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, (free0, free1)
    assert float((back - src).abs().max()) < 1e-2
    print("fresh: ok", free0)
""")


def test_noalloc_allocates_nothing_in_a_fresh_process(env):
    """In a process that never used the pooled path, the entry point runs
    images of new sizes, both directions, on two streams, and the free device
    memory (cudaMemGetInfo) does not move."""
    r = subprocess.run([sys.executable, "-c", _FRESH.format(root=ROOT)], capture_output=True, text=True,
                       timeout=600, env=dict(os.environ, CUDA_MODULE_LOADING="EAGER"))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fresh: ok" in r.stdout
