"""Every frame size from 1 x 1 to 40 x 40, both wavelets, forward then
inverse, bit for bit against the oracle (a stand-in for a sanitizer run,
which is not available on the GPU pool).  Each (size, wavelet) takes one
layout drawn from: the dense frame; an unaligned prime byte row pitch; an
interleaved pixel (stride_y 8 or 12); an outer frame larger than the inner
one, with or without zero padding.  The depth is the full one, 1 or 2, and
decompose_one is drawn too.  Bytes outside the frame, and the samples
between interleaved pixels, must come back untouched."""
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


def _next_prime(n):
    def prime(k):
        return k >= 2 and all(k % d for d in range(2, int(k ** 0.5) + 1))
    while not prime(n):
        n += 1
    return n


def _case(rng, w, h):
    kind = int(rng.integers(0, 4))
    ox, oy, sy, zp = w, h, 4, 0
    if kind == 0:
        sx = 4 * w
    elif kind == 1:
        sx = _next_prime(4 * w + int(rng.integers(1, 17)))
    elif kind == 2:
        sy = int(rng.choice([8, 12]))
        sx = w * sy + 4 * int(rng.integers(0, 3))
    else:
        ox, oy = w + int(rng.integers(0, 9)), h + int(rng.integers(0, 9))
        sx = 4 * ox
        zp = int(rng.integers(0, 2))
    j = int(rng.choice([-1, 1, 2]))
    d1 = int(rng.integers(0, 2))
    return kind, sx, sy, ox, oy, j, d1, zp


def test_every_size_up_to_40(D):
    rng = np.random.default_rng(40)
    bad = []
    for w in range(1, 41):
        for h in range(1, 41):
            for wav in ("cdf97", "cdf53"):
                kind, sx, sy, ox, oy, j, d1, zp = _case(rng, w, h)
                nbytes = sx * (oy - 1) + sy * (ox - 1) + 4 + 16
                buf = rng.integers(0, 256, size=nbytes).astype(np.uint8)
                # the frame's samples: integers 0..255 as floats
                ys, xs = np.meshgrid(np.arange(oy), np.arange(ox), indexing="ij")
                offs = (ys * sx + xs * sy).ravel()
                vals = rng.integers(0, 256, size=offs.size).astype(np.float32).view(np.uint8).reshape(-1, 4)
                for b in range(4):
                    buf[offs + b] = vals[:, b]
                ref = buf.copy()
                got = buf.copy()
                jr = O.transform2(ref, wav, "f", sx, sy, (ox, oy), (w, h), j, d1, zp)
                jg = D.transform2(got, wav, "f", sx, sy, (ox, oy), (w, h), j, d1, zp)
                if jr != jg or not frame_equal(got, ref, sx, sy, ox, oy):
                    bad.append((w, h, wav, kind, sx, sy, ox, oy, j, d1, zp, "f"))
                    continue
                O.transform2(ref, wav, "i", sx, sy, (ox, oy), (w, h), jr, d1, zp)
                D.transform2(got, wav, "i", sx, sy, (ox, oy), (w, h), jr, d1, zp)
                if not frame_equal(got, ref, sx, sy, ox, oy):
                    bad.append((w, h, wav, kind, sx, sy, ox, oy, j, d1, zp, "i"))
    assert not bad, bad[:20]


def test_every_size_up_to_40_on_device_with_guard_bands(D):
    """The same sweep on device frames (dense aligned frames are transformed
    in place by the level kernels, the rest through the repack and unpack
    kernels), each frame between 256-byte guard bands that must come back
    untouched."""
    import torch
    G = 256
    rng = np.random.default_rng(41)
    bad = []
    for w in range(1, 41):
        for h in range(1, 41):
            for wav in ("cdf97", "cdf53"):
                kind, sx, sy, ox, oy, j, d1, zp = _case(rng, w, h)
                nbytes = sx * (oy - 1) + sy * (ox - 1) + 4
                host = rng.integers(0, 256, size=nbytes + 2 * G).astype(np.uint8)
                ys, xs = np.meshgrid(np.arange(oy), np.arange(ox), indexing="ij")
                offs = G + (ys * sx + xs * sy).ravel()
                vals = rng.integers(0, 256, size=offs.size).astype(np.float32).view(np.uint8).reshape(-1, 4)
                for b in range(4):
                    host[offs + b] = vals[:, b]
                ref = host[G:G + nbytes].copy()
                dev = torch.from_numpy(host).cuda()
                frame = dev[G:G + nbytes]
                jr = O.transform2(ref, wav, "f", sx, sy, (ox, oy), (w, h), j, d1, zp)
                jg = D.transform2(frame, wav, "f", sx, sy, (ox, oy), (w, h), j, d1, zp)
                got = dev.cpu().numpy()
                guards_ok = np.array_equal(got[:G], host[:G]) and np.array_equal(got[G + nbytes:], host[G + nbytes:])
                if jr != jg or not guards_ok or not frame_equal(got[G:G + nbytes], ref, sx, sy, ox, oy):
                    bad.append((w, h, wav, kind, sx, sy, ox, oy, j, d1, zp, "f", guards_ok))
                    continue
                O.transform2(ref, wav, "i", sx, sy, (ox, oy), (w, h), jr, d1, zp)
                D.transform2(frame, wav, "i", sx, sy, (ox, oy), (w, h), jr, d1, zp)
                got = dev.cpu().numpy()
                guards_ok = np.array_equal(got[:G], host[:G]) and np.array_equal(got[G + nbytes:], host[G + nbytes:])
                if not guards_ok or not frame_equal(got[G:G + nbytes], ref, sx, sy, ox, oy):
                    bad.append((w, h, wav, kind, sx, sy, ox, oy, j, d1, zp, "i", guards_ok))
    assert not bad, bad[:20]
