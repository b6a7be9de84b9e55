"""The coefficient-layout helpers (dwt_util_subband_s, dwt_util_get_sizes_s /
_d, dwt_util_is_prime / next_prime / get_opt_stride) against the reference's
own results (tests/golden/util.json, made by tests/golden/make_golden_util.py
from the compiled reference).  Host-only functions: no GPU needed."""
import ctypes as C
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def env():
    import libdwt_gb300 as D
    L = D.lib()
    L.dwt_util_subband_s.argtypes = [C.c_void_p] + [C.c_int] * 8 + [C.POINTER(C.c_void_p), C.POINTER(C.c_int),
                                                                     C.POINTER(C.c_int)]
    L.dwt_util_subband_s.restype = None
    for p in ("s", "d"):
        f = getattr(L, f"dwt_util_get_sizes_{p}")
        f.argtypes = [C.c_int] * 4 + [C.POINTER(C.c_int)] * 6
        f.restype = None
    with open(os.path.join(HERE, "golden", "util.json")) as f:
        g = json.load(f)
    return L, g


def test_subband_matches_reference(env):
    L, g = env
    base = g["base"]
    bad = []
    for (sx, sy, ox, oy, ix, iy, j, band, off, w, h) in g["subband"]:
        p, pw, ph = C.c_void_p(), C.c_int(), C.c_int()
        L.dwt_util_subband_s(base, sx, sy, ox, oy, ix, iy, j, band, C.byref(p), C.byref(pw), C.byref(ph))
        got = (int(p.value or 0) - base, pw.value, ph.value)
        if got != (off, w, h):
            bad.append(((sx, sy, ox, oy, ix, iy, j, band), got, (off, w, h)))
    assert not bad, bad[:5]
    assert len(g["subband"]) > 1000


def test_get_sizes_matches_reference(env):
    L, g = env
    for (prec, arr, x, y, opt, *want) in g["get_sizes"]:
        v = [C.c_int() for _ in range(6)]
        getattr(L, f"dwt_util_get_sizes_{prec}")(arr, x, y, opt, *[C.byref(t) for t in v])
        assert [t.value for t in v] == want, (prec, arr, x, y, opt)


def test_primes_match_reference(env):
    L, g = env
    pseudo = 0
    for (n, is_p, nxt, opt) in g["primes"]:
        assert L.dwt_util_is_prime(n) == is_p, n
        if nxt is not None:
            assert L.dwt_util_next_prime(n) == nxt, n
        if opt is not None:
            assert L.dwt_util_get_opt_stride(n) == opt, n
        if is_p and n > 2 and any(n % d == 0 for d in range(3, int(n ** 0.5) + 1, 2)):
            pseudo += 1
    # the reference's Fermat test accepts base-2 pseudoprimes (341, 561, ...)
    assert pseudo >= 3
