"""The oracle is pinned to the reference: bit-exact on every golden vector
(produced by the reference library itself) and, where the reference was
compiled here, on fresh random cases.  CPU only."""
import numpy as np
import pytest

from oracle import oracle as O


def _run_2d(case, inp, impl="oracle"):
    buf = inp.copy()
    j = O.transform2(buf, case["wavelet"], case["direction"], case["stride_x"], case["stride_y"],
                     (case["ox"], case["oy"]), (case["ix"], case["iy"]), case["j"],
                     case["decompose_one"], case["zero_padding"], "s", 1, impl)
    return buf, j


def test_golden_2d(golden):
    cases = golden.cases("2d")
    assert len(cases) > 200
    for c in cases:
        inp, out = golden.io(c)
        got, j = _run_2d(c, inp)
        assert j == c["j_out"], c
        assert np.array_equal(got, out), c


def test_golden_1d(golden):
    for c in golden.cases("1d"):
        inp, out = golden.io(c)
        buf = inp.copy()
        base = buf.ctypes.data
        N, st = c["N"], c["stride"]
        h = base + ((N + 1) // 2) * st
        if c["direction"] == "f":
            O.strided_1d(c["wavelet"], "f", base, base, h, N, st)
        else:
            O.strided_1d(c["wavelet"], "i", base, h, base, N, st)
        assert np.array_equal(buf, out), c


def test_golden_2d_double(golden):
    for c in golden.cases("2d_d"):
        inp, out = golden.io(c)
        got, j = O.transform2_dense(inp, c["wavelet"], c["direction"], c["j"], 0, "d")
        assert j == c["j_out"]
        assert np.array_equal(got, out), c


def test_example_simple_roundtrip(golden):
    """examples/simple/simple.c: test image, forward to full depth, inverse,
    dwt_util_compare_s (absolute 1e-3, src/libdwt.c:1251-1277)."""
    c = golden.cases("example_simple")[0]
    img, out = golden.io(c)
    W, H = c["ox"], c["oy"]
    mine = np.zeros((H, W), np.float32)
    O.test_image_fill_s(mine, W * 4, 4, W, H, 0)
    assert np.array_equal(mine, img)
    fwd, j = O.transform2_dense(img, "cdf97", "f", -1)
    back, _ = O.transform2_dense(fwd, "cdf97", "i", j)
    assert np.array_equal(fwd, out[0]) and np.array_equal(back, out[1])
    assert np.all(np.isfinite(back)) and np.max(np.abs(back - img)) <= 1e-3


@pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")
def test_oracle_vs_reference_random():
    rng = np.random.default_rng(7)
    for _ in range(60):
        ix, iy = int(rng.integers(1, 70)), int(rng.integers(1, 70))
        ox, oy = ix + int(rng.integers(0, 6)), iy + int(rng.integers(0, 6))
        sy = int(rng.choice([4, 12]))
        sx = ox * sy + int(rng.choice([0, 4, 7]))
        c = dict(wavelet=str(rng.choice(["cdf97", "cdf53"])), direction=str(rng.choice(["f", "i"])),
                 stride_x=sx, stride_y=sy, ox=ox, oy=oy, ix=ix, iy=iy, j=int(rng.integers(-1, 8)),
                 decompose_one=int(rng.integers(0, 2)), zero_padding=int(rng.integers(0, 2)))
        # bytes below 0x40: every 4-byte window, aligned or not, is a finite float
        inp = rng.integers(0, 64, size=sx * oy + 16).astype(np.uint8)
        a, ja = _run_2d(c, inp, "oracle")
        b, jb = _run_2d(c, inp, "ref")
        assert ja == jb and np.array_equal(a, b), c


def test_planted_mistake_is_caught(golden):
    """The parity check is sharp: a one-ulp change planted in the oracle's
    output is reported as a mismatch."""
    c = golden.cases("2d")[40]
    inp, out = golden.io(c)
    got, _ = _run_2d(c, inp)
    f = got.view(np.uint8)[: (len(got) // 4) * 4].view(np.float32).copy()
    k = int(np.flatnonzero(f)[0])
    f[k] = np.nextafter(f[k], np.float32(np.inf))
    planted = got.copy()
    planted[: len(f) * 4] = f.view(np.uint8)
    assert not np.array_equal(planted, out)
