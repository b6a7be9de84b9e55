"""ctypes front end of the CPU checker -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/_build/liboracle.so`` (the C restatement in ``dwt_oracle.c``)
and, where it was built, ``oracle/_ref/libdwt_ref.so`` (the reference library
itself, compiled by ``oracle/Makefile``).  Only the tests, the smoke check and
the CPU-baseline leg of ``bench.py`` import this module; the product library
never does.

Every 2D helper takes and returns numpy arrays in the reference's memory model:
a byte buffer, a row stride ``stride_x`` and a pixel stride ``stride_y``, both in
bytes, exactly as ``dwt_cdf97_2f_s`` (src/libdwt.c:6286) receives them.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libdwt_ref.so")

_vp = C.c_void_p
_i = C.c_int


def reference_dir() -> str:
    """Where the reference checkout lies: $DWT_REFERENCE_DIR, else a directory
    named ``reference`` beside this repository (it is read, never written)."""
    d = os.environ.get("DWT_REFERENCE_DIR")
    return d if d else os.path.abspath(os.path.join(HERE, "..", "..", "reference"))


def build(ref: bool = False) -> None:
    """Compile the oracle (and, if asked and its source exists, the reference)."""
    targets = ["oracle"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE, f"REF_DIR={reference_dir()}"] + targets, check=True)


def _declare(lib, prefix: str) -> None:
    for w in ("cdf97", "cdf53"):
        getattr(lib, f"{prefix}{w}_f_ex_stride_s").argtypes = [_vp, _vp, _vp, _vp, _i, _i]
        getattr(lib, f"{prefix}{w}_i_ex_stride_s").argtypes = [_vp, _vp, _vp, _vp, _i, _i]
        getattr(lib, f"{prefix}{w}_f_ex_stride_d").argtypes = [_vp, _vp, _vp, _vp, _i, _i]
        getattr(lib, f"{prefix}{w}_i_ex_stride_d").argtypes = [_vp, _vp, _vp, _vp, _i, _i]


_oracle = None
_ref = None


def lib():
    """The oracle library (built on first use)."""
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(
                os.path.join(HERE, "dwt_oracle.c")):
            build()
        L = C.CDLL(ORACLE_SO)
        _declare(L, "oracle_")
        for w in ("cdf97", "cdf53"):
            for t in ("s", "d"):
                getattr(L, f"oracle_{w}_2f_{t}").argtypes = [_vp, _i, _i, _i, _i, _i, _i,
                                                            C.POINTER(_i), _i, _i, _i]
                getattr(L, f"oracle_{w}_2i_{t}").argtypes = [_vp, _i, _i, _i, _i, _i, _i,
                                                            _i, _i, _i, _i]
        L.oracle_cdf97_1_batch_s.argtypes = [_vp, _i, _i, C.c_long, _i, C.c_long, _i, _i, _i]
        L.oracle_call_1_batch_s.argtypes = [_vp, _vp, _i, _i, C.c_long, _i, C.c_long, _i, _i, _i]
        L.oracle_test_image_fill_s.argtypes = [_vp, _i, _i, _i, _i, _i]
        L.oracle_max_threads.restype = _i
        _oracle = L
    return _oracle


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    """The compiled reference library, or None where it was not built."""
    global _ref
    if _ref is None and ref_available():
        L = C.CDLL(REF_SO)
        _declare(L, "dwt_")
        for w in ("cdf97", "cdf53"):
            for t in ("s", "d"):
                getattr(L, f"dwt_{w}_2f_{t}").argtypes = [_vp, _i, _i, _i, _i, _i, _i,
                                                         C.POINTER(_i), _i, _i]
                getattr(L, f"dwt_{w}_2i_{t}").argtypes = [_vp, _i, _i, _i, _i, _i, _i,
                                                         _i, _i, _i]
        L.dwt_util_set_accel.argtypes = [_i]
        L.dwt_util_set_num_threads.argtypes = [_i]
        _ref = L
    return _ref


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


# ------------------------------------------------------------------ 2D calls

def transform2(buf: np.ndarray, wavelet: str, direction: str, stride_x: int, stride_y: int,
               size_o: tuple, size_i: tuple, j_max: int, decompose_one: int = 0,
               zero_padding: int = 0, precision: str = "s", threads: int = 1,
               impl: str = "oracle") -> int:
    """Run one 2D transform in place on the raw byte buffer ``buf``.

    ``size_o`` = (outer width, outer height), ``size_i`` = (inner width, inner
    height).  Returns the achieved number of levels (what the forward writes back
    through ``j_max_ptr``; for the inverse, the ``j_max`` argument).
    ``impl`` is "oracle" (C restatement) or "ref" (the compiled reference; its
    OpenMP thread count is set through dwt_util_set_num_threads).
    """
    assert buf.flags["C_CONTIGUOUS"]
    ox, oy = size_o
    ix, iy = size_i
    if impl == "oracle":
        L = lib()
        name = f"oracle_{wavelet}_2{direction}_{precision}"
        extra = (threads,)
    else:
        L = ref()
        assert L is not None, "reference library not built"
        L.dwt_util_set_num_threads(max(1, threads))
        name = f"dwt_{wavelet}_2{direction}_{precision}"
        extra = ()
    fn = getattr(L, name)
    if direction == "f":
        j = C.c_int(j_max)
        fn(_ptr(buf), stride_x, stride_y, ox, oy, ix, iy, C.byref(j), decompose_one,
           zero_padding, *extra)
        return j.value
    fn(_ptr(buf), stride_x, stride_y, ox, oy, ix, iy, j_max, decompose_one, zero_padding, *extra)
    return j_max


def transform2_dense(img: np.ndarray, wavelet: str, direction: str, j_max: int,
                     decompose_one: int = 0, precision: str = "s", threads: int = 1,
                     impl: str = "oracle"):
    """Convenience form for a dense row-major image (outer == inner).

    Returns (coefficients as a new array, achieved levels)."""
    dt = np.float32 if precision == "s" else np.float64
    a = np.ascontiguousarray(img, dtype=dt).copy()
    h, w = a.shape
    es = a.itemsize
    j = transform2(a.view(np.uint8).reshape(-1), wavelet, direction, w * es, es, (w, h), (w, h),
                   j_max, decompose_one, 0, precision, threads, impl)
    return a, j


# ------------------------------------------------------------------ 1D calls

def strided_1d(wavelet: str, direction: str, src, dst_a, dst_b, N: int, stride: int,
               precision: str = "s", impl: str = "oracle") -> None:
    """Call ``dwt_<wavelet>_{f,i}_ex_stride_<precision>`` on raw addresses.

    Forward: (src, dst_l, dst_h); inverse: (src_l, src_h, dst)."""
    es = 4 if precision == "s" else 8
    tmp = np.zeros(N + 8, dtype=np.float32 if precision == "s" else np.float64)
    if impl == "oracle":
        fn = getattr(lib(), f"oracle_{wavelet}_{direction}_ex_stride_{precision}")
    else:
        fn = getattr(ref(), f"dwt_{wavelet}_{direction}_ex_stride_{precision}")
    # accel_lift_op4s_s asserts a 16-byte aligned lifting array for some accel
    # values; hand it an aligned temp (forward lifts tmp+1).
    base = _ptr(tmp)
    off = (-(base + (es if direction == "f" else 0))) % 16 // es
    fn(src, dst_a, dst_b, base + off * es, N, stride)


def batch_1d_cdf97(buf: np.ndarray, N: int, stride: int, count: int, group: int,
                   group_stride: int, lane_stride: int, inverse: bool, threads: int = 1) -> None:
    """In-place batched strided CDF 9/7 over ``count`` signals (oracle only)."""
    lib().oracle_cdf97_1_batch_s(_ptr(buf), N, stride, count, group, group_stride, lane_stride,
                                 1 if inverse else 0, threads)


def test_image_fill_s(buf: np.ndarray, stride_x: int, stride_y: int, ix: int, iy: int,
                      rand: int = 0) -> None:
    lib().oracle_test_image_fill_s(_ptr(buf), stride_x, stride_y, ix, iy, rand)
