"""Golden vectors of libdwt's coefficient-layout helpers, by running the
reference library itself.

Run (where the reference source is present):

    make -C oracle ref && python tests/golden/make_golden_util.py

It writes ``tests/golden/util.json``: the results of dwt_util_subband_s
(src/libdwt.c:8153-8262), dwt_util_get_sizes_s / _d (src/libdwt.c:8620-8701)
and dwt_util_is_prime / dwt_util_next_prime / dwt_util_get_opt_stride
(src/libdwt.c:8072-8151) over a grid of inputs, base-2 pseudoprimes
included.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

BASE = 0x100000  # a fake frame address: the helpers only do address arithmetic


def main() -> None:
    assert O.ref_available(), "build the reference first: make -C oracle ref"
    R = O.ref()
    R.dwt_util_subband_s.argtypes = [C.c_void_p] + [C.c_int] * 8 + [C.POINTER(C.c_void_p), C.POINTER(C.c_int),
                                                                     C.POINTER(C.c_int)]
    gs_args = [C.c_int] * 4 + [C.POINTER(C.c_int)] * 6
    R.dwt_util_get_sizes_s.argtypes = gs_args
    R.dwt_util_get_sizes_d.argtypes = gs_args
    out = {"generator": "tests/golden/make_golden_util.py", "base": BASE, "subband": [], "get_sizes": [],
           "primes": []}
    frames = [(1, 1, 1, 1), (7, 5, 7, 5), (8, 8, 8, 8), (33, 47, 33, 47), (64, 64, 33, 47), (128, 64, 100, 37),
              (1024, 1024, 1024, 1024), (1023, 1025, 1023, 1025), (512, 256, 300, 200)]
    for (ox, oy, ix, iy) in frames:
        for sx, sy in [(4 * ox, 4), (4 * ox + 12, 4), (997, 12)]:
            for j in range(0, 12):
                for band in range(4):
                    p, w, h = C.c_void_p(), C.c_int(), C.c_int()
                    R.dwt_util_subband_s(BASE, sx, sy, ox, oy, ix, iy, j, band, C.byref(p), C.byref(w), C.byref(h))
                    out["subband"].append([sx, sy, ox, oy, ix, iy, j, band, int(p.value or 0) - BASE, w.value,
                                           h.value])
    for prec in ("s", "d"):
        fn = getattr(R, f"dwt_util_get_sizes_{prec}")
        for arr in range(3):
            for (x, y) in [(1, 1), (3, 5), (16, 16), (100, 37), (513, 511), (1920, 1080), (4096, 4096)]:
                for opt in (0, 1):
                    v = [C.c_int() for _ in range(6)]
                    fn(arr, x, y, opt, *[C.byref(t) for t in v])
                    out["get_sizes"].append([prec, arr, x, y, opt] + [t.value for t in v])
    for n in list(range(-3, 2200)) + [4095, 4097, 8191, 65537, 65535, 131071, 262145]:
        out["primes"].append([n, R.dwt_util_is_prime(n), R.dwt_util_next_prime(n) if n < 1 << 20 else None,
                              R.dwt_util_get_opt_stride(n) if n > 0 else None])
    with open(os.path.join(HERE, "util.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(len(out["subband"]), "subband cases,", len(out["get_sizes"]), "size cases,", len(out["primes"]), "primes")


if __name__ == "__main__":
    main()
