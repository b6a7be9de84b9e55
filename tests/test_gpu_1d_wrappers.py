"""GPU parity of libdwt's unstrided 1D entry points (src/libdwt.c:1279-1465):
dwt_cdf{97,53}_{f,i}_s (one array: L at [0, ceil(N/2)), H behind it) and
dwt_cdf{97,53}_{f,i}_ex_s (separate L and H arrays), on host and device
memory, for every length 1..24 and a few longer ones, bit for bit against the
oracle's strided restatement called with a 4-byte stride.  Guard samples
around every output must come back untouched."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

LENGTHS = list(range(1, 25)) + [31, 64, 97, 255, 4097]
GUARD = 8


@pytest.fixture(scope="module")
def L():
    import libdwt_gb300 as D
    lib = D.lib()
    for w in ("cdf97", "cdf53"):
        for d in ("f", "i"):
            getattr(lib, f"dwt_{w}_{d}_s").argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
            getattr(lib, f"dwt_{w}_{d}_s").restype = None
            getattr(lib, f"dwt_{w}_{d}_ex_s").argtypes = [C.c_void_p] * 4 + [C.c_int]
            getattr(lib, f"dwt_{w}_{d}_ex_s").restype = None
    return lib


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


def _signal(rng, n):
    return rng.integers(0, 256, size=n).astype(np.float32)


def _oracle_forward(wav, x):
    n = len(x)
    lo = np.zeros((n + 1) // 2, np.float32)
    hi = np.zeros(max(n // 2, 1), np.float32)
    O.strided_1d(wav, "f", x.ctypes.data, lo.ctypes.data, hi.ctypes.data, n, 4)
    return lo, hi[: n // 2]


def _oracle_inverse(wav, lo, hi, n):
    out = np.zeros(n, np.float32)
    hh = hi if len(hi) else np.zeros(1, np.float32)
    O.strided_1d(wav, "i", lo.ctypes.data, hh.ctypes.data, out.ctypes.data, n, 4)
    return out


class _Mem:
    """A float buffer with NaN guard bands on host or device; .ptr(i) is the
    address of sample i of the payload."""

    def __init__(self, torch, n, device):
        self.torch = torch
        self.n = n
        self.t = torch.full((n + 2 * GUARD,), float("nan"), dtype=torch.float32,
                            device="cuda" if device else "cpu")

    def put(self, x):
        self.t[GUARD:GUARD + len(x)] = self.torch.from_numpy(x).to(self.t.device)

    def ptr(self, i=0):
        return self.t.data_ptr() + 4 * (GUARD + i)

    def get(self):
        self.torch.cuda.synchronize()
        a = self.t.cpu().numpy()
        assert np.isnan(a[:GUARD]).all() and np.isnan(a[GUARD + self.n:]).all(), "guard samples overwritten"
        return a[GUARD:GUARD + self.n]


@pytest.mark.parametrize("device", [False, True])
@pytest.mark.parametrize("wav", ["cdf97", "cdf53"])
def test_packed_forward_inverse(L, torch, wav, device):
    rng = np.random.default_rng(101 if wav == "cdf97" else 103)
    f = getattr(L, f"dwt_{wav}_f_s")
    i = getattr(L, f"dwt_{wav}_i_s")
    for n in LENGTHS:
        x = _signal(rng, n)
        lo, hi = _oracle_forward(wav, x)
        src, dst, back = _Mem(torch, n, device), _Mem(torch, n, device), _Mem(torch, n, device)
        src.put(x)
        f(src.ptr(), dst.ptr(), None, n)
        got = dst.get()
        assert np.array_equal(got[: (n + 1) // 2], lo), (wav, n, "L")
        assert np.array_equal(got[(n + 1) // 2:], hi), (wav, n, "H")
        i(dst.ptr(), back.ptr(), None, n)
        assert np.array_equal(back.get(), _oracle_inverse(wav, lo, hi, n)), (wav, n, "inverse")


@pytest.mark.parametrize("device", [False, True])
@pytest.mark.parametrize("wav", ["cdf97", "cdf53"])
def test_split_forward_inverse(L, torch, wav, device):
    rng = np.random.default_rng(107 if wav == "cdf97" else 109)
    f = getattr(L, f"dwt_{wav}_f_ex_s")
    i = getattr(L, f"dwt_{wav}_i_ex_s")
    for n in LENGTHS:
        x = _signal(rng, n)
        lo, hi = _oracle_forward(wav, x)
        nl, nh = (n + 1) // 2, n // 2
        src, ml, mh, back = (_Mem(torch, n, device), _Mem(torch, nl, device), _Mem(torch, max(nh, 1), device),
                             _Mem(torch, n, device))
        src.put(x)
        f(src.ptr(), ml.ptr(), mh.ptr(), None, n)
        got_l = ml.get()
        got_h = mh.get()[:nh]
        assert np.array_equal(got_l, lo), (wav, n, "L")
        assert np.array_equal(got_h, hi), (wav, n, "H")
        if nh == 0:
            assert np.isnan(mh.get()).all(), "N = 1 must not write H"
        i(ml.ptr(), mh.ptr(), back.ptr(), None, n)
        assert np.array_equal(back.get(), _oracle_inverse(wav, lo, hi, n)), (wav, n, "inverse")
