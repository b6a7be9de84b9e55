"""Full-size parity: the 16384 x 16384 and 16383 x 16385 images, CDF 9/7 and
CDF 5/3, forward and inverse to the full depth, bit-exact against the oracle
(the reference's float path), and the error of both against the FP64 path.

Error normalisation (the reference's own float path misses 1e-5 of the input
range on deep forward coefficients, which grow by s1 per level): forward
errors are divided by the range (max - min) of the FP64 coefficients, inverse
errors by the input range 255.  Tolerance 1e-5.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def env():
    import torch

    import libdwt_gb300 as D
    from libdwt_gb300 import synth
    D.lib()
    return D, torch, synth


@pytest.mark.parametrize("size", [(16384, 16384), (16383, 16385)])
def test_fullsize_bit_exact(env, size):
    D, torch, synth = env
    W, H = size
    threads = O.max_threads()
    img = synth.image(W, H, seed=3)
    pw = (W + 3) // 4 * 4
    src = torch.zeros((H, pw), dtype=torch.float32, device="cuda")
    dst = torch.empty((H, W), dtype=torch.float32, device="cuda")
    report = {}
    for wav in ("cdf97", "cdf53"):
        src[:, :W] = torch.from_numpy(img).cuda()
        j = D.transform2_dev(src[:, :W], dst, wav, False, -1)
        torch.cuda.synchronize()
        got_f = dst.cpu().numpy()
        ref_f, jr = O.transform2_dense(img, wav, "f", -1, 0, "s", threads)
        assert j == jr == 14
        assert np.array_equal(got_f, ref_f), f"{wav} forward differs from the oracle"
        src[:, :W] = dst
        D.transform2_dev(src[:, :W], dst, wav, True, j)
        torch.cuda.synchronize()
        got_i = dst.cpu().numpy()
        ref_i, _ = O.transform2_dense(ref_f, wav, "i", j, 0, "s", threads)
        assert np.array_equal(got_i, ref_i), f"{wav} inverse differs from the oracle"
        # FP64 path of the reference on the same input
        d_f, _ = O.transform2_dense(img.astype(np.float64), wav, "f", -1, 0, "d", threads)
        rng = float(d_f.max() - d_f.min())
        ef = np.abs(got_f.astype(np.float64) - d_f)
        d_i, _ = O.transform2_dense(d_f, wav, "i", j, 0, "d", threads)
        ei = np.abs(got_i.astype(np.float64) - d_i)
        rt = np.abs(got_i.astype(np.float64) - img)
        report[wav] = dict(fwd_max=float(ef.max() / rng), fwd_rms=float(np.sqrt((ef ** 2).mean()) / rng),
                           inv_max=float(ei.max() / 255), roundtrip_max=float(rt.max() / 255))
        assert report[wav]["fwd_max"] <= TOL and report[wav]["inv_max"] <= TOL
        assert report[wav]["roundtrip_max"] <= TOL
    print(f"{W}x{H} errors vs FP64: {report}")
