"""Generate golden vectors by running the reference library itself.

Run (where the reference source is present):

    make -C oracle ref && python tests/golden/make_golden.py

It writes ``tests/golden/golden.npz`` (inputs and outputs as raw bytes) and
``tests/golden/golden.json`` (the call parameters of every case).  Each case
is one call of a reference function on a seeded buffer:

* ``2d``: dwt_cdf{97,53}_2{f,i}_s on a byte buffer with the given strides and
  outer/inner frame (src/libdwt.c:6286-6832), including sparse frames with
  zero padding, a prime row pitch in bytes and interleaved pixels;
* ``1d``: dwt_cdf{97,53}_{f,i}_ex_stride_s (src/libdwt.c:5512-5870) for every
  length 1..24 and a few longer ones, in place, unit and interleaved strides;
* ``2d_d``: the double-precision 2D drivers (src/libdwt.c:6120-6645), the
  FP64 reference used for error reporting;
* ``example_simple``: the round trip of examples/simple/simple.c:40-82 on the
  reference test image (dwt_util_test_image_fill_s, src/libdwt.c:1108-1178).

The reference's own tests hold no stored coefficients (it has no test
directory), so these vectors, produced from its source, are the pin.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def main() -> None:
    assert O.ref_available(), "build the reference first: make -C oracle ref"
    rng = np.random.default_rng(20130129)
    cases = []
    arrays = {}

    def add(kind, params, inp: np.ndarray, out: np.ndarray, j_out=None):
        cid = f"c{len(cases):04d}"
        arrays[cid + "_in"] = inp
        arrays[cid + "_out"] = out
        d = {"id": cid, "kind": kind, **params}
        if j_out is not None:
            d["j_out"] = int(j_out)
        cases.append(d)

    # ---- 2D float, dense and sparse frames, both wavelets, both directions
    specs = []
    for (w, h) in [(1, 1), (1, 7), (9, 1), (2, 2), (2, 3), (3, 5), (4, 4), (5, 8), (7, 7),
                   (16, 16), (33, 47), (31, 64), (64, 33)]:
        for j in (-1, 2):
            for d1 in (0, 1):
                specs.append(dict(ix=w, iy=h, ox=w, oy=h, sy=4, pad=0, j=j, d1=d1, zp=0))
    for (w, h) in [(65, 65), (127, 40)]:
        specs.append(dict(ix=w, iy=h, ox=w, oy=h, sy=4, pad=0, j=-1, d1=0, zp=0))
    for _ in range(30):
        ix, iy = int(rng.integers(1, 48)), int(rng.integers(1, 48))
        ox, oy = ix + int(rng.integers(0, 10)), iy + int(rng.integers(0, 10))
        specs.append(dict(ix=ix, iy=iy, ox=ox, oy=oy, sy=int(rng.choice([4, 8, 12])),
                          pad=int(rng.choice([0, 4, 12, 20])), j=int(rng.integers(-1, 6)),
                          d1=int(rng.integers(0, 2)), zp=int(rng.integers(0, 2))))
    # interleaved channels (stride_y = 12, three floats per pixel) and a
    # prime pitch in bytes, the layout dwt_util_get_opt_stride hands out
    specs.append(dict(ix=61, iy=29, ox=61, oy=29, sy=12, pad=0, j=-1, d1=0, zp=0))
    specs.append(dict(ix=50, iy=21, ox=50, oy=21, sy=4, pad=3, j=-1, d1=1, zp=0))
    for sp in specs:
        for wav in ("cdf97", "cdf53"):
            for direc in ("f", "i"):
                sx = sp["ox"] * sp["sy"] + sp["pad"]
                nbytes = sx * sp["oy"] + 16
                inp = rng.integers(0, 256, size=(nbytes + 3) // 4).astype(np.float32)
                inp = inp.view(np.uint8)[:nbytes].copy()
                out = inp.copy()
                jo = O.transform2(out, wav, direc, sx, sp["sy"], (sp["ox"], sp["oy"]),
                                  (sp["ix"], sp["iy"]), sp["j"], sp["d1"], sp["zp"], "s", 1, "ref")
                add("2d", dict(wavelet=wav, direction=direc, stride_x=sx, stride_y=sp["sy"],
                               ox=sp["ox"], oy=sp["oy"], ix=sp["ix"], iy=sp["iy"], j=sp["j"],
                               decompose_one=sp["d1"], zero_padding=sp["zp"]), inp, out, jo)

    # ---- 1D float strided, in place (L first, then H, same stride)
    for wav in ("cdf97", "cdf53"):
        for direc in ("f", "i"):
            for N in list(range(1, 25)) + [31, 32, 63, 100, 257]:
                for st in (4, 12):
                    nbytes = N * st + 16
                    inp = rng.normal(0, 50, size=(nbytes + 3) // 4).astype(np.float32)
                    inp = inp.view(np.uint8)[:nbytes].copy()
                    out = inp.copy()
                    base = out.ctypes.data
                    h = base + ((N + 1) // 2) * st
                    if direc == "f":
                        O.strided_1d(wav, "f", base, base, h, N, st, "s", "ref")
                    else:
                        O.strided_1d(wav, "i", base, h, base, N, st, "s", "ref")
                    add("1d", dict(wavelet=wav, direction=direc, N=N, stride=st), inp, out)

    # ---- 2D double (the FP64 reference)
    for (w, h, j) in [(33, 47, -1), (64, 64, 3), (5, 8, -1)]:
        for wav in ("cdf97", "cdf53"):
            for direc in ("f", "i"):
                img = rng.integers(0, 256, size=(h, w)).astype(np.float64)
                out, jo = O.transform2_dense(img, wav, direc, j, 0, "d", 1, "ref")
                add("2d_d", dict(wavelet=wav, direction=direc, ox=w, oy=h, ix=w, iy=h, j=j,
                                 decompose_one=0), img, out, jo)

    # ---- examples/simple/simple.c: test image, full-depth forward then inverse
    W, H = 97, 63
    img = np.zeros((H, W), np.float32)
    O.test_image_fill_s(img, W * 4, 4, W, H, 0)
    fwd, jo = O.transform2_dense(img, "cdf97", "f", -1, 0, "s", 1, "ref")
    back, _ = O.transform2_dense(fwd, "cdf97", "i", jo, 0, "s", 1, "ref")
    add("example_simple", dict(wavelet="cdf97", ox=W, oy=H, j=-1), img, np.stack([fwd, back]), jo)

    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "reference": "slchen/libdwt 2013-01-29-dev, src/libdwt.c, accel 0",
                   "cases": cases}, f, indent=0)
    print(f"{len(cases)} cases written")


if __name__ == "__main__":
    main()
