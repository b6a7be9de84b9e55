"""libdwt_gb300: GB300-native drop-in for libdwt's lifting wavelet hot path.

The product is the C-ABI shared library ``libdwt_gb300/_lib/libdwt_gb300.so``
(declared in ``include/libdwt.h``).  This module loads it with ctypes and
mirrors the reference's C interface for Python callers: the same function
names and arguments (raw addresses, byte strides, outer/inner frame, j_max,
decompose_one, zero_padding), plus helpers that accept numpy arrays (host
memory) and torch CUDA tensors (device memory).

There is no CPU implementation here: if the library is missing, loading
fails with an error naming the build step.
"""
from __future__ import annotations

import ctypes as C
import os

from .buildext import LIB, build, up_to_date  # noqa: F401

__all__ = ["lib", "build", "CDF97", "CDF53", "DwtError", "transform2", "transform2_dev",
           "strided_1d", "batch_1d"]

CDF97 = 0
CDF53 = 1
_WAVELETS = {"cdf97": CDF97, "cdf53": CDF53, CDF97: CDF97, CDF53: CDF53}

_vp = C.c_void_p
_i = C.c_int
_ll = C.c_longlong


class DwtError(RuntimeError):
    pass


class BatchImage(C.Structure):
    """dwt_gpu_batch_image (include/libdwt.h)."""
    _fields_ = [("src", _vp), ("src_pitch_bytes", _ll), ("dst", _vp), ("dst_pitch_bytes", _ll),
                ("w", _i), ("h", _i), ("j_levels", _i), ("decompose_one", _i), ("wavelet", _i),
                ("inverse", _i)]


class Request(C.Structure):
    """dwt_gpu_request (include/libdwt.h)."""
    _fields_ = [("src", _vp), ("src_pitch_bytes", _ll), ("dst", _vp), ("dst_pitch_bytes", _ll),
                ("w", _i), ("h", _i), ("j_levels", _i), ("decompose_one", _i), ("wavelet", _i),
                ("inverse", _i), ("tag", _ll)]


class Completion(C.Structure):
    """dwt_gpu_completion (include/libdwt.h)."""
    _fields_ = [("id", _ll), ("tag", _ll), ("status", _i), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_complete", C.c_double)]


class ServerStats(C.Structure):
    """dwt_gpu_server_stats_t (include/libdwt.h)."""
    _fields_ = [("submitted", _ll), ("completed", _ll), ("launches", _ll), ("pending", _ll),
                ("bytes_in_use", _ll), ("peak_bytes", _ll), ("budget_bytes", _ll), ("arena_bytes", _ll),
                ("device_allocs", _ll), ("max_dispatch_ns", _ll)]


class BatchParams(C.Structure):
    """dwt_gpu_batch_params (include/libdwt.h)."""
    _fields_ = [("seg_pairs", _i), ("tail_side", _i), ("ctas_per_sm", _i)]


_lib = None


def lib():
    """The loaded CUDA library.  Raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise ImportError(f"libdwt_gb300 CUDA library not built ({LIB}); "
                              "run python -c 'import __graft_entry__ as g; g.build()'")
        L = C.CDLL(LIB)
        for w in ("cdf97", "cdf53"):
            getattr(L, f"dwt_{w}_2f_s").argtypes = [_vp, _i, _i, _i, _i, _i, _i, C.POINTER(_i), _i, _i]
            getattr(L, f"dwt_{w}_2i_s").argtypes = [_vp, _i, _i, _i, _i, _i, _i, _i, _i, _i]
            getattr(L, f"dwt_{w}_f_ex_stride_s").argtypes = [_vp, _vp, _vp, _vp, _i, _i]
            getattr(L, f"dwt_{w}_i_ex_stride_s").argtypes = [_vp, _vp, _vp, _vp, _i, _i]
        L.dwt_util_subband_s.argtypes = [_vp] + [_i] * 8 + [C.POINTER(_vp), C.POINTER(_i), C.POINTER(_i)]
        L.dwt_util_subband_s.restype = None
        L.dwt_util_get_sizes_s.argtypes = [_i] * 4 + [C.POINTER(_i)] * 6
        L.dwt_util_get_sizes_s.restype = None
        L.dwt_gpu_2f_s.argtypes = [_i, _vp, _i, _i, _i, _i, _i, _i, C.POINTER(_i), _i, _i]
        L.dwt_gpu_2i_s.argtypes = [_i, _vp, _i, _i, _i, _i, _i, _i, _i, _i, _i]
        L.dwt_gpu_1_s.argtypes = [_i, _i, _vp, _vp, _vp, _vp, _i, _i]
        L.dwt_gpu_2_channels_s.argtypes = [_i, _i, _vp, _i, _i, _i, _i, C.POINTER(_i), _i]
        L.dwt_gpu_2f_d.argtypes = [_i, _vp, _i, _i, _i, _i, _i, _i, C.POINTER(_i), _i, _i]
        L.dwt_gpu_2i_d.argtypes = [_i, _vp, _i, _i, _i, _i, _i, _i, _i, _i, _i]
        L.dwt_gpu_1_d.argtypes = [_i, _i, _vp, _vp, _vp, _vp, _i, _i]
        L.dwt_gpu_2_dev.argtypes = [_i, _i, _vp, _ll, _vp, _ll, _i, _i, _i, _i, _vp]
        L.dwt_gpu_1_batch_s.argtypes = [_i, _i, _vp, _i, _i, _ll, _i, _ll, _i]
        L.dwt_gpu_level_dev.argtypes = [_i, _i, _i, _i, C.POINTER(_vp), C.POINTER(_ll),
                                        C.POINTER(_vp), C.POINTER(_ll), _vp]
        L.dwt_gpu_batch_create.argtypes = [C.POINTER(C.c_void_p), _i, C.POINTER(BatchImage),
                                           C.POINTER(BatchParams)]
        L.dwt_gpu_batch_run.argtypes = [C.c_void_p, _vp]
        L.dwt_gpu_batch_params_get.argtypes = [C.c_void_p, C.POINTER(BatchParams)]
        L.dwt_gpu_batch_items.argtypes = [C.c_void_p]
        L.dwt_gpu_batch_destroy.argtypes = [C.c_void_p]
        L.dwt_gpu_sync_check.restype = _i
        L.dwt_gpu_server_create.argtypes = [C.POINTER(C.c_void_p), _ll, _i, C.POINTER(BatchParams)]
        L.dwt_gpu_server_reserve.argtypes = [C.c_void_p, _ll]
        L.dwt_gpu_server_submit.argtypes = [C.c_void_p, C.POINTER(Request), C.POINTER(_ll)]
        L.dwt_gpu_server_poll.argtypes = [C.c_void_p, C.POINTER(Completion), _i, C.POINTER(_i)]
        L.dwt_gpu_server_drain.argtypes = [C.c_void_p, C.c_double]
        L.dwt_gpu_server_stats.argtypes = [C.c_void_p, C.POINTER(ServerStats)]
        L.dwt_gpu_server_replay.argtypes = [C.c_void_p, _i, C.POINTER(C.c_double), C.POINTER(Request),
                                            C.POINTER(C.c_double), C.c_double]
        L.dwt_gpu_server_destroy.argtypes = [C.c_void_p]
        L.dwt_gpu_error_string.restype = C.c_char_p
        L.dwt_gpu_error_string.argtypes = [_i]
        L.dwt_util_set_accel.argtypes = [_i]
        L.dwt_util_ceil_log2.argtypes = [_i]
        _lib = L
    return _lib


def _check(rc: int) -> int:
    if rc < 0:
        raise DwtError(lib().dwt_gpu_error_string(rc).decode())
    return rc


def _addr(x) -> int:
    """Address of a numpy array, a torch tensor or an int."""
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return x.ctypes.data


# ------------------------------------------------------------ reference API

def dwt_cdf97_2f_s(ptr, stride_x, stride_y, size_o_big_x, size_o_big_y, size_i_big_x,
                   size_i_big_y, j_max, decompose_one=0, zero_padding=0) -> int:
    """In-place forward CDF 9/7 (src/libdwt.c:6286).  Returns the achieved j_max."""
    j = C.c_int(j_max)
    _check(lib().dwt_gpu_2f_s(CDF97, _addr(ptr), stride_x, stride_y, size_o_big_x, size_o_big_y,
                              size_i_big_x, size_i_big_y, C.byref(j), decompose_one, zero_padding))
    return j.value


def dwt_cdf53_2f_s(ptr, stride_x, stride_y, size_o_big_x, size_o_big_y, size_i_big_x,
                   size_i_big_y, j_max, decompose_one=0, zero_padding=0) -> int:
    """In-place forward CDF 5/3 (src/libdwt.c:6410).  Returns the achieved j_max."""
    j = C.c_int(j_max)
    _check(lib().dwt_gpu_2f_s(CDF53, _addr(ptr), stride_x, stride_y, size_o_big_x, size_o_big_y,
                              size_i_big_x, size_i_big_y, C.byref(j), decompose_one, zero_padding))
    return j.value


def dwt_cdf97_2i_s(ptr, stride_x, stride_y, size_o_big_x, size_o_big_y, size_i_big_x,
                   size_i_big_y, j_max, decompose_one=0, zero_padding=0) -> None:
    """In-place inverse CDF 9/7 (src/libdwt.c:6647)."""
    _check(lib().dwt_gpu_2i_s(CDF97, _addr(ptr), stride_x, stride_y, size_o_big_x, size_o_big_y,
                              size_i_big_x, size_i_big_y, j_max, decompose_one, zero_padding))


def dwt_cdf53_2i_s(ptr, stride_x, stride_y, size_o_big_x, size_o_big_y, size_i_big_x,
                   size_i_big_y, j_max, decompose_one=0, zero_padding=0) -> None:
    """In-place inverse CDF 5/3 (src/libdwt.c:6757)."""
    _check(lib().dwt_gpu_2i_s(CDF53, _addr(ptr), stride_x, stride_y, size_o_big_x, size_o_big_y,
                              size_i_big_x, size_i_big_y, j_max, decompose_one, zero_padding))


def dwt_cdf97_f_ex_stride_s(src, dst_l, dst_h, tmp, N, stride) -> None:
    """Forward CDF 9/7 level of a strided signal (src/libdwt.c:5512)."""
    _check(lib().dwt_gpu_1_s(CDF97, 0, _addr(src), None, _addr(dst_l), _addr(dst_h), N, stride))


def dwt_cdf97_i_ex_stride_s(src_l, src_h, dst, tmp, N, stride) -> None:
    """Inverse CDF 9/7 level of a strided signal (src/libdwt.c:5779)."""
    _check(lib().dwt_gpu_1_s(CDF97, 1, _addr(src_l), _addr(src_h), _addr(dst), None, N, stride))


def dwt_cdf53_f_ex_stride_s(src, dst_l, dst_h, tmp, N, stride) -> None:
    """Forward CDF 5/3 level of a strided signal (src/libdwt.c:5559)."""
    _check(lib().dwt_gpu_1_s(CDF53, 0, _addr(src), None, _addr(dst_l), _addr(dst_h), N, stride))


def dwt_cdf53_i_ex_stride_s(src_l, src_h, dst, tmp, N, stride) -> None:
    """Inverse CDF 5/3 level of a strided signal (src/libdwt.c:5826)."""
    _check(lib().dwt_gpu_1_s(CDF53, 1, _addr(src_l), _addr(src_h), _addr(dst), None, N, stride))


def dwt_util_init() -> None:
    lib().dwt_util_init()


def dwt_util_finish() -> None:
    lib().dwt_util_finish()


def dwt_util_set_accel(accel_type: int) -> None:
    lib().dwt_util_set_accel(accel_type)


# ------------------------------------------------------------ conveniences

DWT_LL, DWT_HL, DWT_LH, DWT_HH = range(4)
DWT_ARR_SIMPLE, DWT_ARR_SPARSE, DWT_ARR_PACKED = range(3)


def dwt_util_subband_s(ptr, stride_x: int, stride_y: int, size_o_big_x: int, size_o_big_y: int,
                       size_i_big_x: int, size_i_big_y: int, j_max: int, band: int):
    """Address (int) and (width, height) of subband `band` (DWT_LL, DWT_HL,
    DWT_LH, DWT_HH) of level j_max in a transformed frame at `ptr`
    (src/libdwt.c:8153-8262)."""
    L = lib()
    p, w, h = C.c_void_p(), C.c_int(), C.c_int()
    L.dwt_util_subband_s(C.c_void_p(_addr(ptr)), stride_x, stride_y, size_o_big_x, size_o_big_y, size_i_big_x,
                         size_i_big_y, j_max, band, C.byref(p), C.byref(w), C.byref(h))
    return int(p.value or 0), w.value, h.value


def dwt_util_get_sizes_s(array_type: int, size_x: int, size_y: int, opt_stride: int):
    """(stride_x, stride_y, size_o_big_x, size_o_big_y, size_i_big_x,
    size_i_big_y) of a float image in layout `array_type`
    (src/libdwt.c:8620-8659)."""
    L = lib()
    v = [C.c_int() for _ in range(6)]
    L.dwt_util_get_sizes_s(array_type, size_x, size_y, opt_stride, *[C.byref(t) for t in v])
    return tuple(t.value for t in v)


def transform2(buf, wavelet, direction: str, stride_x: int, stride_y: int, size_o, size_i,
               j_max: int, decompose_one: int = 0, zero_padding: int = 0) -> int:
    """One in-place 2D transform on a buffer (numpy array = host, torch CUDA
    tensor = device) holding the frame at byte strides.  Returns the achieved
    levels (forward) or the j_max argument (inverse)."""
    w = _WAVELETS[wavelet]
    ox, oy = size_o
    ix, iy = size_i
    if direction == "f":
        j = C.c_int(j_max)
        _check(lib().dwt_gpu_2f_s(w, _addr(buf), stride_x, stride_y, ox, oy, ix, iy, C.byref(j),
                                  decompose_one, zero_padding))
        return j.value
    _check(lib().dwt_gpu_2i_s(w, _addr(buf), stride_x, stride_y, ox, oy, ix, iy, j_max,
                              decompose_one, zero_padding))
    return j_max


def transform2_dev(src, dst, wavelet, inverse: bool, j_levels: int = -1, decompose_one: int = 0,
                   stream: int = 0) -> int:
    """Device-resident out-of-place dense transform of torch CUDA tensors
    src -> dst (2D float32, row pitch = stride(0)).  Asynchronous on `stream`
    (a raw cudaStream_t, 0 = default).  Returns the achieved depth."""
    h, w = src.shape
    return _check(lib().dwt_gpu_2_dev(_WAVELETS[wavelet], 1 if inverse else 0, src.data_ptr(),
                                      src.stride(0) * 4, dst.data_ptr(), dst.stride(0) * 4, w, h,
                                      j_levels, decompose_one, stream))


def level_dev(wavelet, inverse: bool, w: int, h: int, ins, in_pitch_bytes, outs,
              out_pitch_bytes, stream: int = 0) -> None:
    """One out-of-place level on device pointers (see dwt_gpu_level_dev)."""
    def arr(t, vals):
        vals = list(vals) + [0] * (4 - len(vals))
        return (t * 4)(*vals)
    _check(lib().dwt_gpu_level_dev(_WAVELETS[wavelet], 1 if inverse else 0, w, h,
                                   arr(_vp, [_addr(x) for x in ins]), arr(_ll, in_pitch_bytes),
                                   arr(_vp, [_addr(x) for x in outs]), arr(_ll, out_pitch_bytes),
                                   stream))


def transform2_channels(buf, wavelet, inverse: bool, stride_x: int, channels: int, w: int, h: int,
                        j_levels: int = -1, decompose_one: int = 0) -> int:
    """Every channel of a dense interleaved float image in one call
    (dwt_gpu_2_channels_s); returns the levels run."""
    j = C.c_int(j_levels)
    _check(lib().dwt_gpu_2_channels_s(_WAVELETS[wavelet], 1 if inverse else 0, _addr(buf), stride_x, channels, w, h,
                                      C.byref(j), decompose_one))
    return j.value


def transform2_d(buf, wavelet, direction: str, stride_x: int, stride_y: int, size_o, size_i,
                 j_max: int, decompose_one: int = 0, zero_padding: int = 0) -> int:
    """transform2 in double precision (libdwt's _2f_d / _2i_d)."""
    w = _WAVELETS[wavelet]
    ox, oy = size_o
    ix, iy = size_i
    if direction == "f":
        j = C.c_int(j_max)
        _check(lib().dwt_gpu_2f_d(w, _addr(buf), stride_x, stride_y, ox, oy, ix, iy, C.byref(j),
                                  decompose_one, zero_padding))
        return j.value
    _check(lib().dwt_gpu_2i_d(w, _addr(buf), stride_x, stride_y, ox, oy, ix, iy, j_max,
                              decompose_one, zero_padding))
    return j_max


def strided_1d_d(wavelet, inverse: bool, a, b, c, d, N: int, stride: int) -> None:
    """strided_1d in double precision (libdwt's _ex_stride_d)."""
    _check(lib().dwt_gpu_1_d(_WAVELETS[wavelet], 1 if inverse else 0, _addr(a),
                             None if b is None else _addr(b), _addr(c),
                             None if d is None else _addr(d), N, stride))


def strided_1d(wavelet, inverse: bool, a, b, c, d, N: int, stride: int) -> None:
    """Non-aborting strided 1D level on raw addresses / arrays / tensors."""
    _check(lib().dwt_gpu_1_s(_WAVELETS[wavelet], 1 if inverse else 0, _addr(a),
                             None if b is None else _addr(b), _addr(c),
                             None if d is None else _addr(d), N, stride))


def batch_1d(wavelet, inverse: bool, base, N: int, stride: int, count: int, group: int,
             group_stride: int, lane_stride: int) -> None:
    """Batched in-place strided 1D level over a bank of signals."""
    _check(lib().dwt_gpu_1_batch_s(_WAVELETS[wavelet], 1 if inverse else 0, _addr(base), N, stride,
                                   count, group, group_stride, lane_stride))


class Batch:
    """A planned batch of device-resident images (dwt_gpu_batch_*).

    images: list of dicts with src, dst (torch CUDA tensors, 2D float32; src
    rows 16-byte aligned), wavelet, inverse, j_levels (default -1).
    params: (seg_pairs, tail_side, ctas_per_sm) or None to autotune."""

    def __init__(self, images, params=None):
        L = lib()
        arr = (BatchImage * len(images))()
        for k, im in enumerate(images):
            src, dst = im["src"], im["dst"]
            h, w = dst.shape
            arr[k] = BatchImage(src.data_ptr(), src.stride(0) * 4, dst.data_ptr(), dst.stride(0) * 4, w, h,
                                im.get("j_levels", -1), im.get("decompose_one", 0),
                                _WAVELETS[im["wavelet"]], 1 if im.get("inverse") else 0)
        self._keep = images
        self._h = C.c_void_p()
        p = None if params is None else C.byref(BatchParams(*params))
        _check(L.dwt_gpu_batch_create(C.byref(self._h), len(images), arr, p))

    def run(self, stream: int = 0) -> None:
        _check(lib().dwt_gpu_batch_run(self._h, stream))

    @property
    def params(self):
        p = BatchParams()
        _check(lib().dwt_gpu_batch_params_get(self._h, C.byref(p)))
        return (p.seg_pairs, p.tail_side, p.ctas_per_sm)

    @property
    def items(self) -> int:
        return lib().dwt_gpu_batch_items(self._h)

    def close(self) -> None:
        if self._h:
            lib().dwt_gpu_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The continuous-batching server (dwt_gpu_server_*)."""

    def __init__(self, budget_bytes: int, n_streams: int = 4, params=None):
        self._h = C.c_void_p()
        p = None if params is None else C.byref(BatchParams(*params))
        _check(lib().dwt_gpu_server_create(C.byref(self._h), budget_bytes, n_streams, p))

    @staticmethod
    def request(src, dst, wavelet, inverse=False, j_levels=-1, tag=0, w=None, h=None) -> Request:
        """A request on torch CUDA tensors; dst=None lets the server write to a pooled buffer."""
        hh, ww = (dst.shape if dst is not None else src.shape) if w is None else (h, w)
        return Request(src.data_ptr() if hasattr(src, "data_ptr") else src,
                       src.stride(0) * 4 if hasattr(src, "stride") else 0,
                       None if dst is None else dst.data_ptr(), 0 if dst is None else dst.stride(0) * 4,
                       ww, hh, j_levels, 0, _WAVELETS[wavelet], 1 if inverse else 0, tag)

    def reserve(self, nbytes: int) -> None:
        """Reserve the arena and load every kernel (dwt_gpu_server_reserve)."""
        _check(lib().dwt_gpu_server_reserve(self._h, nbytes))

    def submit(self, req: Request) -> int:
        i = _ll()
        _check(lib().dwt_gpu_server_submit(self._h, C.byref(req), C.byref(i)))
        return i.value

    def poll(self, max_n: int = 4096):
        buf = (Completion * max_n)()
        n = _i()
        _check(lib().dwt_gpu_server_poll(self._h, buf, max_n, C.byref(n)))
        return [buf[k] for k in range(n.value)]

    def drain(self, timeout_s: float = 60.0) -> None:
        _check(lib().dwt_gpu_server_drain(self._h, timeout_s))

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().dwt_gpu_server_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def replay(self, arrival_s, reqs, timeout_s: float = 300.0):
        """Submit reqs[i] at arrival_s[i] (real time), drain; returns latencies (s)."""
        import numpy as np
        n = len(reqs)
        arr = (C.c_double * n)(*[float(a) for a in arrival_s])
        rq = (Request * n)(*reqs)
        lat = (C.c_double * n)()
        _check(lib().dwt_gpu_server_replay(self._h, n, arr, rq, lat, timeout_s))
        return np.frombuffer(lat, dtype=np.float64).copy()

    def close(self) -> None:
        if self._h:
            lib().dwt_gpu_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
