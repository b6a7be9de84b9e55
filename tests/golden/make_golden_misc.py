"""Golden vectors of libdwt's remaining public utilities, by running the
reference library itself, and the list of functions its public header
declares.

Run (where the reference source is present):

    make -C oracle ref && python tests/golden/make_golden_misc.py

It writes ``tests/golden/misc.json``:

* ``api_functions``: every function name declared in src/libdwt.h;
* ``zero_padding``: buffers after dwt_zero_padding_{f,i}_stride_{s,d}
  (src/libdwt.c:5906-6004) over a grid of lengths and strides;
* ``pgm``: the files dwt_util_save_to_pgm_s / _d (src/libdwt.c:7532-7668)
  write for a small frame with values inside, above and below the range;
* ``conv_show``: the bits dwt_util_conv_show_s / _d (src/libdwt.c:8326-8384)
  produce for a strided frame;
* ``vec``: return codes of the vector helpers (src/libdwt.c:7716-7833);
* ``log``: what dwt_util_log (src/libdwt.c:7953-7985) writes for each level.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

REF_HEADER = os.path.join(O.reference_dir(), "src", "libdwt.h")


def api_functions() -> list:
    text = open(REF_HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    return sorted(set(re.findall(r"\b(dwt_\w+)\s*\(", text)))


def pgm_frame(dtype):
    # 5 x 4 frame inside a 7-float row pitch: in range, above max, below 0
    ox, oy, pitch = 5, 4, 7
    a = np.full((oy, pitch), -7.0, dtype=dtype)
    vals = np.array([0.0, 0.5, 1.0, 0.999, 0.0004, 1.0005, 1.01, -0.0005, -0.5, 0.25,
                     0.3333, 0.6667, 2.0, 1e-7, 0.123456, 0.75, 0.9, 0.1, 0.01, 0.001], dtype=dtype)
    a[:, :ox] = vals.reshape(oy, ox)
    return a, ox, oy, pitch


def main() -> None:
    assert O.ref_available(), "build the reference first: make -C oracle ref"
    R = O.ref()
    out = {"generator": "tests/golden/make_golden_misc.py", "api_functions": api_functions(),
           "zero_padding": [], "pgm": {}, "conv_show": {}, "vec": {}, "log": {}}

    # zero padding
    for t, ct, dt in (("s", C.c_float, np.float32), ("d", C.c_double, np.float64)):
        es = np.dtype(dt).itemsize
        fwd = getattr(R, f"dwt_zero_padding_f_stride_{t}")
        fwd.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        inv = getattr(R, f"dwt_zero_padding_i_stride_{t}")
        inv.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
        for N in (0, 1, 2, 3, 7, 8, 13):
            for extra in (0, 1, 2, 3):
                nl, nh = (N + 1) // 2 + extra, N // 2 + extra + ((N & 1) if extra else 0)
                if (nl - nh) & ~1:
                    continue  # outside the reference's precondition
                for step in (1, 3):
                    stride = step * es
                    buf = np.arange(1, 1 + 2 * 24 * step, dtype=dt)
                    base = buf.ctypes.data
                    fwd(base, base + 24 * step * es, N, nl, nh, stride)
                    out["zero_padding"].append({"t": t, "dir": "f", "N": N, "nl": nl, "nh": nh, "stride": stride,
                                                "out": buf.tolist()})
                    buf = np.arange(1, 1 + 24 * step, dtype=dt)
                    inv(buf.ctypes.data, N, N + extra, stride)
                    out["zero_padding"].append({"t": t, "dir": "i", "N": N, "nd": N + extra, "stride": stride,
                                                "out": buf.tolist()})

    # PGM files (the warnings go to stderr and are not recorded)
    for t, ct, dt in (("s", C.c_float, np.float32), ("d", C.c_double, np.float64)):
        fn = getattr(R, f"dwt_util_save_to_pgm_{t}")
        fn.argtypes = [C.c_char_p, ct, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        a, ox, oy, pitch = pgm_frame(dt)
        es = np.dtype(dt).itemsize
        for mx in (1.0, 0.5, 3.0):
            with tempfile.TemporaryDirectory() as d:
                path = os.path.join(d, "x.pgm")
                rc = fn(path.encode(), mx, a.ctypes.data, pitch * es, es, ox, oy)
                out["pgm"][f"{t}_{mx}"] = {"rc": rc, "text": open(path).read(), "frame": a.tolist(),
                                           "ox": ox, "oy": oy}

    # log-magnitude view of a strided frame
    rng = np.random.default_rng(7)
    for t, dt, it in (("s", np.float32, np.uint32), ("d", np.float64, np.uint64)):
        fn = getattr(R, f"dwt_util_conv_show_{t}")
        fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        src = (rng.standard_normal((9, 13)) * np.array([1e-3, 1, 1e3])[rng.integers(0, 3, (9, 13))]).astype(dt)
        src[0, :4] = [0.0, -0.0, 1e-30, -2.5]
        dst = np.full_like(src, 5.0)
        es = np.dtype(dt).itemsize
        fn(src.ctypes.data, dst.ctypes.data, 13 * es, 2 * es, 6, 9)  # every other column
        out["conv_show"][t] = {"src": src.view(it).tolist(), "dst": dst.view(it).tolist()}

    # vector helpers
    R.dwt_util_generate_vec_s.argtypes = [C.c_void_p, C.c_int]
    R.dwt_util_zero_vec_s.argtypes = [C.c_void_p, C.c_int]
    R.dwt_util_copy_vec_s.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    R.dwt_util_cmp_vec_s.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    v = np.zeros(64, np.float32)
    w = np.zeros(64, np.float32)
    out["vec"]["generate"] = [R.dwt_util_generate_vec_s(v.ctypes.data, 64), v.tolist()]
    out["vec"]["copy"] = [R.dwt_util_copy_vec_s(v.ctypes.data, w.ctypes.data, 64), w.tolist()]
    cmp_cases = []
    # (kind, position, value): "add" perturbs b[pos] by value, "set" stores it
    for kind, pos, val in (("add", 0, 0.0), ("add", 3, 5e-5), ("add", 3, 2e-4), ("set", 10, "inf"),
                           ("set", 63, "nan"), ("set", 0, 1e-40)):
        a = np.arange(64, dtype=np.float32)
        b = a.copy()
        x = np.float32(float(val))
        b[pos] = b[pos] + x if kind == "add" else x
        cmp_cases.append([kind, pos, val, R.dwt_util_cmp_vec_s(a.ctypes.data, b.ctypes.data, 64)])
    out["vec"]["cmp"] = cmp_cases
    out["vec"]["zero"] = R.dwt_util_zero_vec_s(v.ctypes.data, 64)

    # log lines, captured from a child process
    code = ("import ctypes as C, sys; L = C.CDLL(sys.argv[1]); "
            "[L.dwt_util_log(l, b'level %d: %s %.3f\\n', l, b'msg', C.c_double(1.5)) for l in range(6)]")
    r = subprocess.run([sys.executable, "-c", code, O.REF_SO], capture_output=True, check=True)
    out["log"]["stderr"] = r.stderr.decode()

    with open(os.path.join(HERE, "misc.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(len(out["api_functions"]), "functions,", len(out["zero_padding"]), "padding cases")


if __name__ == "__main__":
    main()
