"""GPU parity: every output of the CUDA path, called through the C ABI,
equals the reference's float path bit for bit (golden vectors produced by the
reference, and the oracle that is pinned to it)."""
import numpy as np
import pytest

from conftest import frame_equal
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def D():
    import libdwt_gb300
    libdwt_gb300.lib()
    return libdwt_gb300


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


def _gpu_2d(D, buf, c, j):
    return D.transform2(buf, c["wavelet"], c["direction"], c["stride_x"], c["stride_y"],
                        (c["ox"], c["oy"]), (c["ix"], c["iy"]), j, c["decompose_one"],
                        c["zero_padding"])


def _same(got, exp, c):
    return frame_equal(got, exp, c["stride_x"], c["stride_y"], c["ox"], c["oy"])


def test_golden_2d_host(D, golden):
    bad = []
    for c in golden.cases("2d"):
        inp, out = golden.io(c)
        buf = inp.copy()
        j = _gpu_2d(D, buf, c, c["j"])
        if (c["direction"] == "f" and j != c["j_out"]) or not _same(buf, out, c):
            bad.append(c)
    assert not bad, f"{len(bad)} mismatching cases, first: {bad[:5]}"


def test_golden_2d_device(D, golden, torch):
    bad = []
    for c in golden.cases("2d"):
        inp, out = golden.io(c)
        dev = torch.from_numpy(inp.copy()).cuda()
        j = _gpu_2d(D, dev, c, c["j"])
        if (c["direction"] == "f" and j != c["j_out"]) or not _same(dev.cpu().numpy(), out, c):
            bad.append(c)
    assert not bad, f"{len(bad)} mismatching cases, first: {bad[:5]}"


def test_golden_1d(D, golden, torch):
    bad = []
    for c in golden.cases("1d"):
        inp, out = golden.io(c)
        N, st = c["N"], c["stride"]
        for where in ("host", "device"):
            if where == "host":
                buf = inp.copy()
                base = buf.ctypes.data
            else:
                t = torch.from_numpy(inp.copy()).cuda()
                base = t.data_ptr()
            h = base + ((N + 1) // 2) * st
            if c["direction"] == "f":
                D.strided_1d(c["wavelet"], False, base, None, base, h, N, st)
            else:
                D.strided_1d(c["wavelet"], True, base, h, base, None, N, st)
            got = buf if where == "host" else t.cpu().numpy()
            if not np.array_equal(got, out):
                bad.append((c, where))
    assert not bad, f"{len(bad)} mismatching cases, first: {bad[:5]}"


def test_random_dense_vs_oracle(D, torch):
    rng = np.random.default_rng(11)
    sizes = [(1, 1), (1, 2), (2, 1), (3, 3), (5, 4), (8, 8), (119, 7), (120, 9), (121, 33), (128, 128),
             (240, 17), (241, 241), (255, 3), (300, 500), (1023, 1025), (17, 1000)]
    bad = []
    for (w, h) in sizes:
        img = rng.integers(0, 256, size=(h, w)).astype(np.float32)
        for wav in ("cdf97", "cdf53"):
            for d1 in (0, 1):
                ref_f, j = O.transform2_dense(img, wav, "f", -1, d1)
                ref_i, _ = O.transform2_dense(ref_f, wav, "i", j, d1)
                dev = torch.from_numpy(img).cuda()
                jj = D.transform2(dev, wav, "f", w * 4, 4, (w, h), (w, h), -1, d1)
                if jj != j or not np.array_equal(dev.cpu().numpy(), ref_f):
                    bad.append((w, h, wav, d1, "f"))
                dev = torch.from_numpy(ref_f).cuda()
                D.transform2(dev, wav, "i", w * 4, 4, (w, h), (w, h), j, d1)
                if not np.array_equal(dev.cpu().numpy(), ref_i):
                    bad.append((w, h, wav, d1, "i"))
    assert not bad, bad


def test_device_out_of_place(D, torch):
    rng = np.random.default_rng(12)
    for (w, h) in [(129, 77), (1000, 600), (4, 3)]:
        img = rng.integers(0, 256, size=(h, w)).astype(np.float32)
        for wav in ("cdf97", "cdf53"):
            ref_f, j = O.transform2_dense(img, wav, "f", -1)
            ref_i, _ = O.transform2_dense(ref_f, wav, "i", j)
            pw = (w + 3) // 4 * 4
            src = torch.zeros((h, pw), dtype=torch.float32, device="cuda")
            src[:, :w] = torch.from_numpy(img).cuda()
            dst = torch.zeros((h, w), dtype=torch.float32, device="cuda")
            jj = D.transform2_dev(src[:, :w], dst, wav, False, -1)
            torch.cuda.synchronize()
            assert jj == j and np.array_equal(dst.cpu().numpy(), ref_f)
            src[:, :w] = dst
            D.transform2_dev(src[:, :w], dst, wav, True, j)
            torch.cuda.synchronize()
            assert np.array_equal(dst.cpu().numpy(), ref_i)


def test_batch_1d_vs_oracle(D, torch):
    """Bank of strided signals (8 interleaved per group, stride 32 B), in place."""
    rng = np.random.default_rng(13)
    N, group, count = 4097, 8, 8 * 37
    groups = count // group
    x = rng.normal(size=(groups, N, group)).astype(np.float32)
    gs, ls, st = N * group * 4, 4, group * 4
    ref = x.copy()
    O.batch_1d_cdf97(ref, N, st, count, group, gs, ls, False, O.max_threads())
    dev = torch.from_numpy(x).cuda()
    D.batch_1d("cdf97", False, dev, N, st, count, group, gs, ls)
    assert np.array_equal(dev.cpu().numpy(), ref)
    ref_i = ref.copy()
    O.batch_1d_cdf97(ref_i, N, st, count, group, gs, ls, True, O.max_threads())
    D.batch_1d("cdf97", True, dev, N, st, count, group, gs, ls)
    assert np.array_equal(dev.cpu().numpy(), ref_i)
    host = ref.copy()
    D.batch_1d("cdf97", True, host, N, st, count, group, gs, ls)
    assert np.array_equal(host, ref_i)


def test_roundtrip_within_reference_tolerance(D, torch):
    """examples/simple/simple.c: forward to full depth, inverse, compare with
    absolute eps 1e-3 (dwt_util_compare_s, src/libdwt.c:1251-1277)."""
    W, H = 1920, 1080
    img = np.zeros((H, W), np.float32)
    O.test_image_fill_s(img, W * 4, 4, W, H, 0)
    for wav in ("cdf97", "cdf53"):
        buf = img.copy()
        j = D.transform2(buf, wav, "f", W * 4, 4, (W, H), (W, H), -1)
        D.transform2(buf, wav, "i", W * 4, 4, (W, H), (W, H), j)
        assert np.all(np.isfinite(buf)) and np.abs(buf - img).max() <= 1e-3


def test_large_host_frames_pipelined(D, torch):
    """Host frames of 4 Mpx and more take the banded copy/compute pipeline;
    outputs stay bit-identical to the oracle (pinned and pageable memory)."""
    rng = np.random.default_rng(17)
    for (w, h, pinned) in [(2500, 2000, True), (2049, 2051, False), (4096, 1024, True), (8192, 601, True),
                           (1031, 4099, True)]:
        img = rng.integers(0, 256, size=(h, w)).astype(np.float32)
        for wav in ("cdf97", "cdf53"):
            for j in (-1, 1, 2, 3):
                ref_f, jr = O.transform2_dense(img, wav, "f", j, 0, "s", O.max_threads())
                ref_i, _ = O.transform2_dense(ref_f, wav, "i", jr, 0, "s", O.max_threads())
                buf = torch.from_numpy(img.copy())
                if pinned:
                    buf = buf.pin_memory()
                arr = buf.numpy()
                jj = D.transform2(arr, wav, "f", w * 4, 4, (w, h), (w, h), j)
                assert jj == jr
                assert np.array_equal(arr, ref_f), (w, h, wav, j, "f")
                D.transform2(arr, wav, "i", w * 4, 4, (w, h), (w, h), jr)
                assert np.array_equal(arr, ref_i), (w, h, wav, j, "i")
