"""dwt_gpu_2_dev_noalloc, the entry point for callers that may not allocate
device memory (its scratch is a fixed array inside the library): called
through the C ABI, its output must equal the regular dwt_gpu_2_dev's bit for
bit, on two calls in a row (the array keeps the first call's contents), and
an image too large for the array must be refused without running.

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

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
