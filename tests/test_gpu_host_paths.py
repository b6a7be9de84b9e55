"""Host frames in pageable memory reach the GPU two ways: copy kernels that
address the caller's memory through the host page tables (where the GPU
supports that), or the copy engines.  Both must give the reference's bits,
for the banded pipeline (4 Mpx and more), the single-shot path, and
byte-strided frames.  The way is chosen once per process
(DWT_GPU_DIRECT_HOST=0 forces the copy engines), so each runs in a child."""
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import libdwt_gb300 as D
w, h, sy, wav, j, src, dst = int(sys.argv[2]), int(sys.argv[3]), int(sys.argv[4]), sys.argv[5], int(sys.argv[6]), sys.argv[7], sys.argv[8]
img = np.load(src)
ch = sy // 4
buf = np.zeros((h, w * ch), np.float32)
buf[:, ::ch] = img
jj = D.transform2(buf, wav, "f", w * sy, sy, (w, h), (w, h), j)
fwd = buf[:, ::ch].copy()
D.transform2(buf, wav, "i", w * sy, sy, (w, h), (w, h), jj)
np.savez(dst, fwd=fwd, inv=buf[:, ::ch].copy(), rest=buf[:, 1::ch] if ch > 1 else np.zeros(1, np.float32), j=jj)
"""


@pytest.mark.parametrize("direct", ["1", "0"])
@pytest.mark.parametrize("w,h,sy,wav", [(2500, 2000, 4, "cdf97"), (2049, 2051, 4, "cdf53"), (301, 203, 4, "cdf97"),
                                        (257, 129, 12, "cdf53")])
def test_pageable_host_frames(tmp_path, direct, w, h, sy, wav):
    rng = np.random.default_rng(w + h)
    img = rng.integers(0, 256, size=(h, w)).astype(np.float32)
    src, dst = str(tmp_path / "in.npy"), str(tmp_path / "out.npz")
    np.save(src, img)
    env = dict(os.environ, DWT_GPU_DIRECT_HOST=direct)
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, str(w), str(h), str(sy), wav, "-1", src, dst],
                       capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr
    out = np.load(dst)
    ref_f, jr = O.transform2_dense(img, wav, "f", -1, 0, "s", O.max_threads())
    ref_i, _ = O.transform2_dense(ref_f, wav, "i", jr, 0, "s", O.max_threads())
    assert int(out["j"]) == jr
    assert np.array_equal(out["fwd"], ref_f)
    assert np.array_equal(out["inv"], ref_i)
    if sy > 4:
        assert not out["rest"].any()  # samples between the pixels are untouched


CHILD_1D = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import libdwt_gb300 as D
N, k, wav, src, dst = int(sys.argv[2]), int(sys.argv[3]), sys.argv[4], sys.argv[5], sys.argv[6]
x = np.load(src)                          # N samples, every k-th float of a host buffer
buf = np.zeros(N * k + 8, np.float32)
buf[:N * k:k] = x
a = buf.copy()
D.strided_1d(wav, False, a, None, a, a[(N + 1) // 2 * k:], N, 4 * k)   # in place: L then H
fwd = a.copy()
D.strided_1d(wav, True, a, a[(N + 1) // 2 * k:], a, None, N, 4 * k)
np.savez(dst, fwd=fwd, inv=a)
"""


@pytest.mark.parametrize("direct", ["1", "0"])
@pytest.mark.parametrize("N,k,wav", [(1, 1, "cdf97"), (2, 8, "cdf53"), (7, 3, "cdf97"), (4097, 8, "cdf97"),
                                     (1000, 1, "cdf53")])
def test_pageable_1d_signals(tmp_path, direct, N, k, wav):
    rng = np.random.default_rng(N + k)
    x = rng.standard_normal(N).astype(np.float32)
    src, dst = str(tmp_path / "x.npy"), str(tmp_path / "o.npz")
    np.save(src, x)
    env = dict(os.environ, DWT_GPU_DIRECT_HOST=direct)
    r = subprocess.run([sys.executable, "-c", CHILD_1D, ROOT, str(N), str(k), wav, src, dst], capture_output=True,
                       text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    out = np.load(dst)
    buf = np.zeros(N * k + 8, np.float32)
    buf[:N * k:k] = x
    ref = buf.copy()
    base = ref.ctypes.data
    hoff = (N + 1) // 2 * k * 4
    O.strided_1d(wav, "f", base, base, base + hoff, N, 4 * k)
    assert np.array_equal(out["fwd"], ref)
    O.strided_1d(wav, "i", base, base + hoff, base, N, 4 * k)
    assert np.array_equal(out["inv"], ref)
