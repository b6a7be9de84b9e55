"""Interleaved multi-channel images in one call (dwt_gpu_2_channels_s)
against the reference's way, one drop-in call per channel with
stride_y = 4 * channels (src/cvdwt.cpp:67-147): bit-identical results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    import libdwt_gb300 as D
    D.lib()
    return D, torch


@pytest.mark.parametrize("shape", [(131, 257, 3), (97, 64, 4), (33, 1000, 3), (1, 40, 2)])
@pytest.mark.parametrize("wav", ["cdf97", "cdf53"])
def test_channels_match_per_channel_calls(env, shape, wav):
    D, torch = env
    h, w, ch = shape
    rng = np.random.default_rng(h * w * ch)
    pad = 3 * ch  # a row stride larger than the row
    img = np.zeros((h, (w + pad) * ch), np.float32)
    img[:, : w * ch] = rng.integers(0, 256, size=(h, w * ch))
    sx = img.shape[1] * 4
    for d1 in (0, 1):
        for inverse in (False, True):
            want = img.copy()
            js = []
            for c in range(ch):
                base = want.ctypes.data + 4 * c
                if inverse:
                    D.transform2(base, wav, "i", sx, 4 * ch, (w, h), (w, h), -1, d1)
                else:
                    js.append(D.transform2(base, wav, "f", sx, 4 * ch, (w, h), (w, h), -1, d1))
            for where in ("host", "device"):
                if where == "host":
                    got = img.copy()
                    j = D.transform2_channels(got, wav, inverse, sx, ch, w, h, -1, d1)
                else:
                    t = torch.from_numpy(img.copy()).cuda()
                    j = D.transform2_channels(t, wav, inverse, sx, ch, w, h, -1, d1)
                    torch.cuda.synchronize()
                    got = t.cpu().numpy()
                if not inverse:
                    assert j == js[0]
                assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (where, inverse, d1)
