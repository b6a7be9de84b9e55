"""Frames past 2^31 samples: every offset the kernels and the host paths form
must be 64-bit.  A 46344 x 46341 image (2,147,627,304 samples, 8.6 GB; rows
16-byte aligned, as the device form requires, and an odd height) is
transformed on the device and through the pageable host path; level-1 rows
at the top and the bottom of the frame (sample offsets beyond 2^31) are
compared bit for bit with the oracle run on a band of rows that contains
them, and the host path must reproduce the device path.  The strided 1D
drop-in takes a single signal of 2^27 + 3 samples."""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

W, H = 46344, 46341
assert W * H > 2 ** 31


@pytest.fixture(scope="module")
def D():
    import libdwt_gb300
    libdwt_gb300.lib()
    return libdwt_gb300


@pytest.fixture(scope="module")
def big(D):
    import torch
    free, _ = torch.cuda.mem_get_info()
    if free < 40 * 2 ** 30:
        pytest.skip("needs 40 GiB of free device memory")
    torch.manual_seed(5)
    src = torch.empty(H, W, device="cuda").random_(0, 256)
    dst = torch.empty_like(src)
    s = torch.cuda.current_stream().cuda_stream
    assert D.transform2_dev(src, dst, "cdf97", False, 1, 0, s) == 1
    torch.cuda.synchronize()
    yield torch, src, dst
    del src, dst
    torch.cuda.empty_cache()


def _check_rows(src, dst, r0, r1):
    """Oracle level 1 on source rows [2*r0, 2*r1) (whole width); pairs more
    than 4 away from a cut edge of that band are exact."""
    hd = (H + 1) // 2
    hh = H // 2
    lo, hi = 2 * r0, min(H, 2 * r1)
    sub = src[lo:hi].cpu().numpy()
    ref, _ = O.transform2_dense(sub, "cdf97", "f", 1, 0, "s", O.max_threads())
    hs_sub = (hi - lo + 1) // 2
    p_lo = r0 if r0 == 0 else r0 + 4
    p_hi = min(hd, r1) if hi == H else r1 - 4
    got_top = dst[p_lo:p_hi].cpu().numpy()                       # LL | HL rows
    assert np.array_equal(got_top, ref[p_lo - r0:p_hi - r0])
    q_hi = min(p_hi, hh)
    got_bot = dst[hd + p_lo:hd + q_hi].cpu().numpy()            # LH | HH rows
    assert np.array_equal(got_bot, ref[hs_sub + p_lo - r0:hs_sub + q_hi - r0])


def test_device_level1_rows_at_both_ends(big):
    torch, src, dst = big
    hd = (H + 1) // 2
    _check_rows(src, dst, 0, 16)
    _check_rows(src, dst, hd - 16, hd)  # LH/HH rows near the end: offsets > 2^31 samples
    _check_rows(src, dst, hd // 2 - 8, hd // 2 + 8)


def test_device_full_depth_round_trip(big, D):
    torch, src, _ = big
    s = torch.cuda.current_stream().cuda_stream
    coef = torch.empty_like(src)
    j = D.transform2_dev(src, coef, "cdf97", False, -1, 0, s)
    rec = torch.empty_like(src)
    D.transform2_dev(coef, rec, "cdf97", True, j, 0, s)
    torch.cuda.synchronize()
    err = (rec - src).abs().max().item()
    assert j == 16 and err <= 5e-3, (j, err)  # 2e-5 of the input range
    del coef, rec


def test_pageable_host_frame_matches_device(big, D):
    torch, src, dst = big
    avail = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    if avail < 32 * 2 ** 30:
        pytest.skip("needs 32 GiB of free host memory")
    img = src.cpu().numpy()                     # pageable, 8.6 GB
    assert D.transform2(img, "cdf97", "f", W * 4, 4, (W, H), (W, H), 1) == 1
    step = 2048
    for r in range(0, H, step):
        assert np.array_equal(img[r:r + step], dst[r:r + step].cpu().numpy()), r
    s = torch.cuda.current_stream().cuda_stream
    rec = torch.empty_like(src)
    D.transform2_dev(dst, rec, "cdf97", True, 1, 0, s)
    torch.cuda.synchronize()
    D.transform2(img, "cdf97", "i", W * 4, 4, (W, H), (W, H), 1)
    for r in range(0, H, step):
        assert np.array_equal(img[r:r + step], rec[r:r + step].cpu().numpy()), r
    del rec, img


def test_strided_1d_signal_of_2_27_samples(D):
    N = 2 ** 27 + 3
    rng = np.random.default_rng(9)
    x = rng.standard_normal(N).astype(np.float32)
    a = x.copy()
    hoff = (N + 1) // 2
    D.strided_1d("cdf97", False, a, None, a, a[hoff:], N, 4)
    ref = x.copy()
    base = ref.ctypes.data
    O.strided_1d("cdf97", "f", base, base, base + hoff * 4, N, 4)
    assert np.array_equal(a, ref)
    D.strided_1d("cdf97", True, a, a[hoff:], a, None, N, 4)
    O.strided_1d("cdf97", "i", base, base + hoff * 4, base, N, 4)
    assert np.array_equal(a, ref)
