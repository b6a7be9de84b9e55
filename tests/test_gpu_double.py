"""Double precision (libdwt's _d API) on the GPU: bit-exact against the
reference's own double 2D results (the golden 2d_d cases) and against the
oracle's double restatement (src/libdwt.c:1467-1571, 5673-5777, 6120-6645)
on sparse, strided, interleaved and odd frames and on 1D signals."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def D():
    import libdwt_gb300 as D
    D.lib()
    return D


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


def test_golden_2d_d(D, golden):
    bad = []
    cases = golden.cases("2d_d")
    assert cases
    for c in cases:
        inp, out = golden.io(c)
        buf = np.ascontiguousarray(inp.copy())
        h, w = buf.shape
        j = D.transform2_d(buf, c["wavelet"], c["direction"], w * 8, 8, (c["ox"], c["oy"]), (c["ix"], c["iy"]),
                           c["j"], c["decompose_one"])
        if (c["direction"] == "f" and j != c["j_out"]) or not np.array_equal(buf.view(np.uint64),
                                                                            out.view(np.uint64)):
            bad.append(c["id"])
    assert not bad, bad


FRAMES = [
    # ox, oy, ix, iy, stride_x, stride_y, j, decompose_one, zero_padding
    (33, 47, 33, 47, 33 * 8, 8, -1, 0, 0),
    (64, 40, 64, 40, 64 * 8 + 40, 8, 3, 0, 0),
    (17, 9, 17, 9, 17 * 24 + 16, 24, -1, 1, 0),     # interleaved samples
    (29, 31, 29, 31, 241, 8, 2, 0, 0),              # a prime pitch: unaligned doubles
    (64, 64, 37, 50, 64 * 8, 8, 4, 0, 0),           # sparse frame
    (64, 64, 37, 50, 64 * 8, 8, 4, 0, 1),           # sparse frame, zero padding
    (1, 13, 1, 13, 8, 8, -1, 1, 0),
    (5, 1, 5, 1, 40, 8, -1, 1, 0),
]


@pytest.mark.parametrize("frame", FRAMES)
@pytest.mark.parametrize("wav", ["cdf97", "cdf53"])
def test_2d_d_vs_oracle(D, torch, frame, wav):
    ox, oy, ix, iy, sx, sy, j, d1, zp = frame
    rng = np.random.default_rng(ox * 1000 + oy)
    span = (oy - 1) * sx + (ox - 1) * sy + 8
    raw = rng.integers(0, 256, size=span + 24, dtype=np.uint8)
    # fill the samples with values of the benchmark's range
    for y in range(oy):
        for x in range(ox):
            o = y * sx + x * sy
            raw[o:o + 8] = np.frombuffer(np.float64(rng.integers(0, 256)).tobytes(), np.uint8)
    for where in ("host", "device"):
        ref = raw.copy()
        jr = O.transform2(ref, wav, "f", sx, sy, (ox, oy), (ix, iy), j, d1, zp, "d")
        if where == "host":
            got = raw.copy()
            jg = D.transform2_d(got, wav, "f", sx, sy, (ox, oy), (ix, iy), j, d1, zp)
        else:
            t = torch.from_numpy(raw.copy()).cuda()
            jg = D.transform2_d(t, wav, "f", sx, sy, (ox, oy), (ix, iy), j, d1, zp)
            torch.cuda.synchronize()
            got = t.cpu().numpy()
        assert jg == jr
        assert np.array_equal(got, ref), f"forward {where} differs"
        ref_i = ref.copy()
        O.transform2(ref_i, wav, "i", sx, sy, (ox, oy), (ix, iy), jr, d1, zp, "d")
        if where == "host":
            D.transform2_d(got, wav, "i", sx, sy, (ox, oy), (ix, iy), jr, d1, zp)
            got_i = got
        else:
            t = torch.from_numpy(ref.copy()).cuda()
            D.transform2_d(t, wav, "i", sx, sy, (ox, oy), (ix, iy), jr, d1, zp)
            torch.cuda.synchronize()
            got_i = t.cpu().numpy()
        assert np.array_equal(got_i, ref_i), f"inverse {where} differs"


@pytest.mark.parametrize("N", list(range(1, 20)) + [33, 257, 1000])
def test_1d_d_vs_oracle(D, torch, N):
    rng = np.random.default_rng(N)
    nl = (N + 1) // 2
    for wav in ("cdf97", "cdf53"):
        for stride in (8, 24):
            raw = np.zeros(N * stride // 8 + 4, np.float64)
            raw[: N * stride // 8: stride // 8] = rng.standard_normal(N) * 100
            for where in ("host", "device"):
                ref = raw.copy()
                rb = ref.ctypes.data
                O.strided_1d(wav, "f", rb, rb, rb + nl * stride, N, stride, precision="d")
                if where == "host":
                    got = raw.copy()
                    gb = got.ctypes.data
                    D.strided_1d_d(wav, False, gb, None, gb, gb + nl * stride, N, stride)
                else:
                    t = torch.from_numpy(raw.copy()).cuda()
                    gb = t.data_ptr()
                    D.strided_1d_d(wav, False, gb, None, gb, gb + nl * stride, N, stride)
                    torch.cuda.synchronize()
                    got = t.cpu().numpy()
                assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), (wav, stride, where, "f")
                ref_i = ref.copy()
                rb = ref_i.ctypes.data
                O.strided_1d(wav, "i", rb, rb + nl * stride, rb, N, stride, precision="d")
                if where == "host":
                    got_i = ref.copy()
                    gb = got_i.ctypes.data
                    D.strided_1d_d(wav, True, gb, gb + nl * stride, gb, None, N, stride)
                else:
                    t = torch.from_numpy(ref.copy()).cuda()
                    gb = t.data_ptr()
                    D.strided_1d_d(wav, True, gb, gb + nl * stride, gb, None, N, stride)
                    torch.cuda.synchronize()
                    got_i = t.cpu().numpy()
                assert np.array_equal(got_i.view(np.uint64), ref_i.view(np.uint64)), (wav, stride, where, "i")
