"""Sparse frames (outer > inner) with zero padding on the fused path: the
drop-in calls on host and device frames, both wavelets, forward then inverse,
bit-exact against the oracle (the reference's in-place level sequence,
src/libdwt.c:6330-6397 and 6677-6745), with stale samples outside the inner
image and every byte outside the outer frame untouched; and a 12000^2 image
in a 16384^2 frame (the OpenCV wrapper's power-of-two padding)."""
import numpy as np
import pytest

from conftest import frame_equal
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    import libdwt_gb300 as D
    D.lib()
    return D, torch


GEOMS = [
    # (ox, oy, ix, iy, pitch floats, j)
    (512, 512, 300, 280, 512, -1),
    (1024, 768, 1000, 700, 1028, -1),
    (640, 480, 637, 479, 640, 3),
    (2048, 1024, 1500, 1000, 2048, 1),
    (4096, 256, 4000, 250, 4100, -1),
    (512, 512, 20, 400, 516, -1),
    (300, 300, 299, 210, 301, -1),  # pitch not a multiple of 16 bytes (device frames staged)
]


def _oracle(buf, wav, direction, pitch, geom, j):
    ox, oy, ix, iy = geom[:4]
    a = buf.copy()
    jj = O.transform2(a.view(np.uint8).reshape(-1), wav, direction, pitch * 4, 4, (ox, oy), (ix, iy), j, 0, 1,
                      "s", O.max_threads())
    return a, jj


@pytest.mark.parametrize("where", ["host", "device"])
@pytest.mark.parametrize("wav", ["cdf97", "cdf53"])
@pytest.mark.parametrize("geom", GEOMS)
def test_sparse_fused_matches_oracle(env, geom, wav, where):
    D, torch = env
    ox, oy, ix, iy, pitch, j = geom
    rng = np.random.default_rng(ox + 3 * oy + 5 * ix + 7 * iy)
    rows = oy + 1  # one guard row below the frame
    frame = rng.uniform(-20, 280, size=(rows, pitch)).astype(np.float32)
    frame[:iy, :ix] = rng.integers(0, 256, size=(iy, ix))
    ref_f, jr = _oracle(frame, wav, "f", pitch, geom, j)
    if where == "host":
        buf = frame.copy()
        jj = D.transform2(buf, wav, "f", pitch * 4, 4, (ox, oy), (ix, iy), j, 0, 1)
        got_f = buf
    else:
        dev = torch.from_numpy(frame.copy()).cuda()
        jj = D.transform2(dev, wav, "f", pitch * 4, 4, (ox, oy), (ix, iy), j, 0, 1)
        got_f = dev.cpu().numpy()
    assert jj == jr
    assert frame_equal(got_f.view(np.uint8).reshape(-1), ref_f.view(np.uint8).reshape(-1), pitch * 4, 4, ox, oy), \
        f"{geom} {wav} forward differs"
    ref_i, _ = _oracle(ref_f, wav, "i", pitch, geom, jj)
    if where == "host":
        buf = ref_f.copy()
        D.transform2(buf, wav, "i", pitch * 4, 4, (ox, oy), (ix, iy), jj, 0, 1)
        got_i = buf
    else:
        dev = torch.from_numpy(ref_f.copy()).cuda()
        D.transform2(dev, wav, "i", pitch * 4, 4, (ox, oy), (ix, iy), jj, 0, 1)
        got_i = dev.cpu().numpy()
    assert frame_equal(got_i.view(np.uint8).reshape(-1), ref_i.view(np.uint8).reshape(-1), pitch * 4, 4, ox, oy), \
        f"{geom} {wav} inverse differs"


def test_sparse_fused_12000_in_16384(env):
    D, torch = env
    from libdwt_gb300 import synth
    ox = oy = 16384
    ix = iy = 12000
    img = synth.image(ix, iy, seed=9)
    frame = np.zeros((oy, ox), np.float32)
    frame[:iy, :ix] = img
    dev = torch.from_numpy(frame).cuda()
    threads = O.max_threads()
    ref = frame.copy()
    jr = O.transform2(ref.view(np.uint8).reshape(-1), "cdf97", "f", ox * 4, 4, (ox, oy), (ix, iy), -1, 0, 1, "s",
                      threads)
    j = D.transform2(dev, "cdf97", "f", ox * 4, 4, (ox, oy), (ix, iy), -1, 0, 1)
    assert j == jr == 14
    assert np.array_equal(dev.cpu().numpy(), ref)
    O.transform2(ref.view(np.uint8).reshape(-1), "cdf97", "i", ox * 4, 4, (ox, oy), (ix, iy), j, 0, 1, "s", threads)
    D.transform2(dev, "cdf97", "i", ox * 4, 4, (ox, oy), (ix, iy), j, 0, 1)
    assert np.array_equal(dev.cpu().numpy(), ref)
