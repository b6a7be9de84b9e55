"""Drop-in calls from several host threads at once (libdwt's calls are
reentrant; here they share one context): every thread's results stay
bit-identical to the oracle, for host and device images of different sizes,
both wavelets and both directions, 2D and strided 1D, and the per-thread
error code of the non-aborting forms is kept apart."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def D():
    import libdwt_gb300
    libdwt_gb300.lib()
    return libdwt_gb300


def _job(D, torch, k):
    rng = np.random.default_rng(100 + k)
    w, h = [(257, 129), (1024, 768), (2500, 2000), (33, 47), (640, 480), (1500, 1501)][k % 6]
    wav = ("cdf97", "cdf53")[k % 2]
    img = rng.integers(0, 256, size=(h, w)).astype(np.float32)
    ref_f, j = O.transform2_dense(img, wav, "f", -1)
    ref_i, _ = O.transform2_dense(ref_f, wav, "i", j)
    on_device = k % 3 == 2
    buf = torch.from_numpy(img.copy()).cuda() if on_device else img.copy()
    for _ in range(3):
        b = buf.clone() if on_device else buf.copy()
        jj = D.transform2(b, wav, "f", w * 4, 4, (w, h), (w, h), -1)
        got_f = b.cpu().numpy() if on_device else b.copy()
        D.transform2(b, wav, "i", w * 4, 4, (w, h), (w, h), jj)
        got_i = b.cpu().numpy() if on_device else b
        if jj != j or not np.array_equal(got_f, ref_f) or not np.array_equal(got_i, ref_i):
            return f"job {k}: 2D {wav} {w}x{h} differs"
    # a strided 1D signal
    n = 4097 - k
    x = rng.standard_normal(n * 2 + 8).astype(np.float32)
    a, r = x.copy(), x.copy()
    hoff = (n + 1) // 2 * 2
    D.strided_1d(wav, False, a, None, a, a[hoff:], n, 8)
    O.strided_1d(wav, "f", r.ctypes.data, r.ctypes.data, r.ctypes.data + hoff * 4, n, 8)
    if not np.array_equal(a, r):
        return f"job {k}: 1D {wav} n={n} differs"
    return None


def test_concurrent_drop_in_calls(D):
    import torch
    with ThreadPoolExecutor(max_workers=8) as ex:
        errors = [e for e in ex.map(lambda k: _job(D, torch, k), range(24)) if e]
    assert not errors, errors


def test_error_codes_are_per_thread(D):
    import ctypes as C
    L = D.lib()
    L.dwt_gpu_get_last_error.restype = C.c_int

    def bad(_):
        # a negative stride is refused with an error code, in this thread only
        rc = L.dwt_gpu_1_s(0, 0, C.c_void_p(16), None, C.c_void_p(16), C.c_void_p(32), 8, -4)
        return rc, L.dwt_gpu_get_last_error()

    def good(_):
        x = np.ones(64, np.float32)
        D.strided_1d("cdf97", False, x, None, x, x[32:], 64, 4)
        return L.dwt_gpu_get_last_error()

    with ThreadPoolExecutor(max_workers=4) as ex:
        bads = list(ex.map(bad, range(8)))
        goods = list(ex.map(good, range(8)))
    assert all(rc < 0 and last == rc for rc, last in bads)
    assert all(g == 0 for g in goods)
