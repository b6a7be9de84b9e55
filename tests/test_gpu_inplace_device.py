"""The drop-in 2D calls (dwt_cdf{97,53}_2{f,i}_s) on dense device frames of
1 Mpx and more, which run in place with level 0 as one ordered launch that
stages only the HL quadrant and the last segments of its order: bit-exact against the oracle for square, odd and pitched frames,
every sample of a row's padding (pitch > width) untouched, and the same on the
full-size 16384 x 16384 image."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    import libdwt_gb300 as D
    from libdwt_gb300 import synth
    D.lib()
    return D, torch, synth


CASES = [
    # (W, H, pitch in floats, j_max, wavelet)
    (1024, 1024, 1024, 5, "cdf97"),
    (1024, 1024, 1024, -1, "cdf53"),
    (1531, 1023, 1532, -1, "cdf97"),
    (2047, 2049, 2052, -1, "cdf53"),
    (1500, 1400, 1504, 3, "cdf97"),
    (1500, 1400, 1501, -1, "cdf97"),  # pitch not a multiple of 16 bytes: the staged path
    (4096, 257, 4096, -1, "cdf53"),
    (3001, 700, 3004, 2, "cdf53"),
]


@pytest.mark.parametrize("W,H,pitch,j,wav", CASES)
def test_inplace_device_matches_oracle(env, W, H, pitch, j, wav):
    D, torch, synth = env
    threads = O.max_threads()
    img = synth.image(W, H, seed=W + H)
    framed = np.full((H, pitch), -7.0, dtype=np.float32)
    framed[:, :W] = img
    dev = torch.from_numpy(framed).cuda()
    jj = D.transform2(dev, wav, "f", pitch * 4, 4, (W, H), (W, H), j)
    got_f = dev.cpu().numpy()
    ref_f, jr = O.transform2_dense(img, wav, "f", j, 0, "s", threads)
    assert jj == jr
    assert np.array_equal(got_f[:, :W], ref_f), f"{W}x{H} {wav} forward differs"
    assert (got_f[:, W:] == -7.0).all(), "row padding written"
    D.transform2(dev, wav, "i", pitch * 4, 4, (W, H), (W, H), jj)
    got_i = dev.cpu().numpy()
    ref_i, _ = O.transform2_dense(ref_f, wav, "i", jj, 0, "s", threads)
    assert np.array_equal(got_i[:, :W], ref_i), f"{W}x{H} {wav} inverse differs"
    assert (got_i[:, W:] == -7.0).all(), "row padding written"


def test_inplace_device_fullsize(env):
    D, torch, synth = env
    threads = O.max_threads()
    W = H = 16384
    img = synth.image(W, H, seed=5)
    dev = torch.from_numpy(img).cuda()
    for wav in ("cdf97", "cdf53"):
        dev.copy_(torch.from_numpy(img))
        j = D.transform2(dev, wav, "f", W * 4, 4, (W, H), (W, H), -1)
        ref_f, jr = O.transform2_dense(img, wav, "f", -1, 0, "s", threads)
        assert j == jr == 14
        assert np.array_equal(dev.cpu().numpy(), ref_f), f"{wav} forward differs"
        D.transform2(dev, wav, "i", W * 4, 4, (W, H), (W, H), j)
        ref_i, _ = O.transform2_dense(ref_f, wav, "i", j, 0, "s", threads)
        assert np.array_equal(dev.cpu().numpy(), ref_i), f"{wav} inverse differs"


def test_inplace_device_leads():
    """The same frames with no lead and with a long one before the ordered
    level 0's staged segments (DWT_GPU_INPLACE_LEAD, read once per process:
    child processes)."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
            "import numpy as np, torch, libdwt_gb300 as D\n"
            "from libdwt_gb300 import synth\n"
            "import test_gpu_inplace_device as T\n"
            "env = (D, torch, synth)\n"
            "for c in T.CASES[:5]: T.test_inplace_device_matches_oracle(env, *c)\n"
            "print('leads ok')\n") % (root, os.path.join(root, "tests"))
    for lead in ("0", "40"):
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=900,
                           env=dict(os.environ, DWT_GPU_INPLACE_LEAD=lead))
        assert r.returncode == 0 and "leads ok" in r.stdout, r.stdout + r.stderr
