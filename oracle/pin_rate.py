"""Rate pin of the CPU baseline -- TEST INFRASTRUCTURE ONLY.

The GPU machine has no reference source, so its CPU baseline times the oracle's
C restatement (oracle/dwt_oracle.c, bit-exact with the reference).  This
script, run where the reference was compiled from its own source
(oracle/_ref/libdwt_ref.so, `make -C oracle ref`), times the reference itself
at accel 9 -- the SSE shifted double-loop kernels the reference's callers
select with dwt_util_set_accel(9), src/libdwt.c:3439-4097, dispatched at
5379-5510 -- against the oracle on the same images with the same OpenMP
thread count, minimum over loops as dwt_util_perf_cdf97_2_s measures
(src/libdwt.c:8440-8492), and prints one JSON object: per configuration the
two rates and their ratio (reference / oracle).

    python oracle/pin_rate.py [--threads N] [--loops K] [--quick]

Configurations: the 1024^2 plain drop-in (j = 5) with each wavelet, the
16384^2 image (j = 14, 9/7 and 5/3), the 16383 x 16385 odd size (j = 14), all
forward and inverse; and the strided 1D bank (65536 signals of 4097
samples, 8 interleaved per group) through the reference's own calling
pattern, an OpenMP loop of dwt_cdf97_{f,i}_ex_stride_s calls
(oracle_call_1_batch_s).  Inputs are the seeded synthetic images of the
benchmark (libdwt_gb300/synth.py).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# run as a script, this directory comes first on the path and would shadow
# the oracle package with its oracle.py module
sys.path = [p for p in sys.path if os.path.abspath(p or ".") != HERE]
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402


def _best(fn, loops: int) -> float:
    best = float("inf")
    for _ in range(loops):
        t = time.perf_counter()
        fn()
        best = min(best, time.perf_counter() - t)
    return best


def time_2d(img, wavelet, j, impl, threads, loops):
    """Best seconds of one forward and of one inverse transform."""
    if impl == "ref":
        O.ref().dwt_util_set_accel(9)
    work = {}

    def fwd():
        work["f"] = O.transform2_dense(img, wavelet, "f", j, 0, "s", threads, impl)

    tf = _best(fwd, loops)
    coef, jj = work["f"]

    def inv():
        O.transform2_dense(coef, wavelet, "i", jj, 0, "s", threads, impl)

    ti = _best(inv, loops)
    return tf, ti, coef


def time_c4(threads, loops, groups=8192, n=4097, lanes=8):
    from libdwt_gb300 import synth
    x = synth.ar1_bank(groups, n, lanes, seed=4)
    L = O.lib()
    R = O.ref()
    R.dwt_util_set_accel(9)
    gs, st, count = n * lanes * 4, lanes * 4, groups * lanes
    out = {}
    for impl, lib_, pre in (("ref", R, "dwt_"), ("oracle", L, "oracle_")):
        fns = [C.cast(getattr(lib_, f"{pre}cdf97_{d}_ex_stride_s"), C.c_void_p).value for d in ("f", "i")]
        buf = x.copy()
        res = {}
        for inverse in (0, 1):
            res["inv" if inverse else "fwd"] = _best(
                lambda: L.oracle_call_1_batch_s(fns[inverse], buf.ctypes.data, n, st, count, lanes, gs, 4,
                                                inverse, threads), loops)
        out[impl] = res
    samples = count * n
    return {k: {d: round(samples / v[d] / 1e9, 3) for d in v} for k, v in out.items()}, samples


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=O.max_threads())
    ap.add_argument("--loops", type=int, default=5)
    ap.add_argument("--quick", action="store_true", help="skip the 16384^2 and 16383x16385 cases")
    args = ap.parse_args()
    if not O.ref_available():
        raise SystemExit("the reference was not built here (make -C oracle ref)")
    from libdwt_gb300 import synth
    cases = [("c0_1024_cdf97_j5", 1024, 1024, "cdf97", 5), ("c0_1024_cdf53_j5", 1024, 1024, "cdf53", 5)]
    if not args.quick:
        cases += [("c1_16384_cdf97_j14", 16384, 16384, "cdf97", 14),
                  ("c1_16384_cdf53_j14", 16384, 16384, "cdf53", 14),
                  ("c1_16383x16385_cdf97_j14", 16383, 16385, "cdf97", 14),
                  ("c1_16383x16385_cdf53_j14", 16383, 16385, "cdf53", 14)]
    res = {"host": platform.machine(), "cpu": platform.processor() or platform.machine(),
           "threads": args.threads, "loops": args.loops, "accel": 9, "unit": "Mpx/s (inner pixels / best time)",
           "configs": {}}
    for name, w, h, wav, j in cases:
        img = synth.image(w, h, seed=0 if w == h else 1)
        loops = args.loops if w * h <= 4096 * 4096 else max(2, args.loops // 2)
        rf, ri, rc = time_2d(img, wav, j, "ref", args.threads, loops)
        of, oi, oc = time_2d(img, wav, j, "oracle", args.threads, loops)
        px = w * h
        res["configs"][name] = {
            "ref_fwd": round(px / rf / 1e6, 1), "ref_inv": round(px / ri / 1e6, 1),
            "oracle_fwd": round(px / of / 1e6, 1), "oracle_inv": round(px / oi / 1e6, 1),
            "ratio_ref_over_oracle": round((of + oi) / (rf + ri), 3),
            "bit_identical": bool(np.array_equal(rc.view(np.uint32), oc.view(np.uint32)))}
        print(name, res["configs"][name], file=sys.stderr, flush=True)
    c4, samples = time_c4(args.threads, args.loops)
    res["c4_65536x4097_stride32"] = {"unit": "Gsamples/s", **c4,
                                     "ratio_ref_over_oracle_fwd": round(c4["ref"]["fwd"] / c4["oracle"]["fwd"], 3),
                                     "ratio_ref_over_oracle_inv": round(c4["ref"]["inv"] / c4["oracle"]["inv"], 3)}
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
