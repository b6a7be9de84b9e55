"""The rest of libdwt's public C API (zero padding as stand-alone calls,
coefficient addressing, PGM export, the log-magnitude view, vector helpers,
logging, platform queries) against golden vectors made by running the
reference library (tests/golden/make_golden_misc.py).  The display-transform
vectors were made on x86-64 with glibc's logf/log, which this suite's CPU
run shares."""
import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = json.load(open(os.path.join(ROOT, "tests", "golden", "misc.json")))


@pytest.fixture(scope="module")
def lib():
    from libdwt_gb300.buildext import build
    path = build()
    L = C.CDLL(path)
    for t, ct in (("s", C.c_float), ("d", C.c_double)):
        getattr(L, f"dwt_zero_padding_f_stride_{t}").argtypes = [C.c_void_p, C.c_void_p] + [C.c_int] * 4
        getattr(L, f"dwt_zero_padding_i_stride_{t}").argtypes = [C.c_void_p] + [C.c_int] * 3
        getattr(L, f"dwt_zero_padding_f_{t}").argtypes = [C.c_void_p, C.c_void_p] + [C.c_int] * 3
        getattr(L, f"dwt_zero_padding_i_{t}").argtypes = [C.c_void_p] + [C.c_int] * 2
        getattr(L, f"dwt_util_save_to_pgm_{t}").argtypes = [C.c_char_p, ct, C.c_void_p] + [C.c_int] * 4
        getattr(L, f"dwt_util_conv_show_{t}").argtypes = [C.c_void_p, C.c_void_p] + [C.c_int] * 4
    for name in ("dwt_util_addr_coeff", "dwt_util_addr_coeff_s", "dwt_util_addr_coeff_d"):
        getattr(L, name).argtypes = [C.c_void_p] + [C.c_int] * 4
        getattr(L, name).restype = C.c_void_p
    for name in ("dwt_util_version", "dwt_util_arch", "dwt_util_node", "dwt_util_appname"):
        getattr(L, name).restype = C.c_char_p
    L.dwt_util_allocate_vec_s.restype = C.c_void_p
    L.dwt_util_allocate_vec_s.argtypes = [C.c_int]
    L.dwt_util_generate_vec_s.argtypes = [C.c_void_p, C.c_int]
    L.dwt_util_zero_vec_s.argtypes = [C.c_void_p, C.c_int]
    L.dwt_util_copy_vec_s.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    L.dwt_util_cmp_vec_s.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    L.dwt_util_is_aligned_8.argtypes = [C.c_void_p]
    L.dwt_util_test_image_zero_s.argtypes = [C.c_void_p] + [C.c_int] * 4
    return L, path


def test_every_reference_function_is_exported(lib):
    L, path = lib
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines()}
    missing = [f for f in GOLDEN["api_functions"] if f not in exported]
    assert not missing, missing
    assert len(GOLDEN["api_functions"]) >= 100


@pytest.mark.parametrize("case", range(len(GOLDEN["zero_padding"])))
def test_zero_padding_matches_reference(lib, case):
    L, _ = lib
    g = GOLDEN["zero_padding"][case]
    dt = np.float32 if g["t"] == "s" else np.float64
    n = len(g["out"])
    buf = np.arange(1, 1 + n, dtype=dt)
    base = buf.ctypes.data
    es = buf.itemsize
    if g["dir"] == "f":
        getattr(L, f"dwt_zero_padding_f_stride_{g['t']}")(base, base + n // 2 * es, g["N"], g["nl"], g["nh"],
                                                          g["stride"])
    else:
        getattr(L, f"dwt_zero_padding_i_stride_{g['t']}")(base, g["N"], g["nd"], g["stride"])
    np.testing.assert_array_equal(buf, np.array(g["out"], dtype=dt))


def test_unstrided_zero_padding_forms(lib):
    L, _ = lib
    for t, dt in (("s", np.float32), ("d", np.float64)):
        lo = np.ones(8, dt)
        hi = np.ones(8, dt)
        getattr(L, f"dwt_zero_padding_f_{t}")(lo.ctypes.data, hi.ctypes.data, 5, 5, 5)
        np.testing.assert_array_equal(lo, [1, 1, 1, 0, 0, 1, 1, 1])
        np.testing.assert_array_equal(hi, [1, 1, 0, 0, 0, 1, 1, 1])
        v = np.ones(8, dt)
        getattr(L, f"dwt_zero_padding_i_{t}")(v.ctypes.data, 3, 6)
        np.testing.assert_array_equal(v, [1, 1, 1, 0, 0, 0, 1, 1])
        # a destination shorter than its half writes nothing
        v = np.ones(8, dt)
        getattr(L, f"dwt_zero_padding_i_{t}")(v.ctypes.data, 6, 3)
        np.testing.assert_array_equal(v, np.ones(8))


@pytest.mark.parametrize("key", sorted(GOLDEN["pgm"]))
def test_pgm_matches_reference(lib, key, tmp_path):
    L, _ = lib
    g = GOLDEN["pgm"][key]
    t, mx = key.split("_")
    a = np.array(g["frame"], dtype=np.float32 if t == "s" else np.float64)
    ox, oy, pitch = g["ox"], g["oy"], a.shape[1]
    path = str(tmp_path / "x.pgm")
    es = a.itemsize
    rc = getattr(L, f"dwt_util_save_to_pgm_{t}")(path.encode(), float(mx), a.ctypes.data, pitch * es, es, ox, oy)
    assert rc == GOLDEN["pgm"][key]["rc"] == 0
    assert open(path).read() == GOLDEN["pgm"][key]["text"]


def test_pgm_unwritable_path_returns_1(lib):
    L, _ = lib
    a = np.zeros(4, np.float32)
    assert L.dwt_util_save_to_pgm_s(b"/nonexistent-dir/x.pgm", 1.0, a.ctypes.data, 8, 4, 2, 2) == 1


@pytest.mark.parametrize("t", ["s", "d"])
def test_conv_show_matches_reference_bits(lib, t):
    L, _ = lib
    dt, it = (np.float32, np.uint32) if t == "s" else (np.float64, np.uint64)
    g = GOLDEN["conv_show"][t]
    src = np.array(g["src"], dtype=it).view(dt)
    dst = np.full_like(src, 5.0)
    es = src.itemsize
    getattr(L, f"dwt_util_conv_show_{t}")(src.ctypes.data, dst.ctypes.data, 13 * es, 2 * es, 6, 9)
    np.testing.assert_array_equal(dst.view(it), np.array(g["dst"], dtype=it))


def test_vector_helpers(lib):
    L, _ = lib
    p = L.dwt_util_allocate_vec_s(64)
    assert p and p % 8 == 0 and L.dwt_util_is_aligned_8(p) == 1
    assert L.dwt_util_is_aligned_8(p + 4) == 0
    v = np.zeros(64, np.float32)
    w = np.zeros(64, np.float32)
    rc, vals = GOLDEN["vec"]["generate"]
    assert L.dwt_util_generate_vec_s(v.ctypes.data, 64) == rc
    np.testing.assert_array_equal(v, vals)
    rc, vals = GOLDEN["vec"]["copy"]
    assert L.dwt_util_copy_vec_s(v.ctypes.data, w.ctypes.data, 64) == rc
    np.testing.assert_array_equal(w, vals)
    for kind, pos, val, rc in GOLDEN["vec"]["cmp"]:
        a = np.arange(64, dtype=np.float32)
        b = a.copy()
        x = np.float32(float(val))
        b[pos] = b[pos] + x if kind == "add" else x
        assert L.dwt_util_cmp_vec_s(a.ctypes.data, b.ctypes.data, 64) == rc, (kind, pos, val)
    assert L.dwt_util_zero_vec_s(v.ctypes.data, 64) == GOLDEN["vec"]["zero"]
    assert not v.any()


def test_addressing_and_image_zero(lib):
    L, _ = lib
    for name in ("dwt_util_addr_coeff", "dwt_util_addr_coeff_s", "dwt_util_addr_coeff_d"):
        assert getattr(L, name)(0x10000, 3, 5, 1000, 12) == 0x10000 + 3 * 1000 + 5 * 12
    img = np.ones((4, 6), np.float32)
    L.dwt_util_test_image_zero_s(img.ctypes.data, 24, 8, 3, 2)  # every other column, 2 rows
    exp = np.ones((4, 6), np.float32)
    exp[:2, 0:6:2] = 0
    np.testing.assert_array_equal(img, exp)


def _run_child(code, path):
    return subprocess.run([sys.executable, "-c", code, path], capture_output=True, timeout=120)


def test_log_lines_match_reference(lib):
    _, path = lib
    code = ("import ctypes as C, sys; L = C.CDLL(sys.argv[1]); "
            "[L.dwt_util_log(l, b'level %d: %s %.3f\\n', l, b'msg', C.c_double(1.5)) for l in range(6)]")
    r = _run_child(code, path)
    assert r.returncode == 0
    assert r.stderr.decode() == GOLDEN["log"]["stderr"]


def test_printf_wrappers(lib):
    _, path = lib
    code = ("import ctypes as C, sys; L = C.CDLL(sys.argv[1]); "
            "n = L.dwt_util_printf(b'%s=%d\\n', b'x', 42); C.CDLL(None).fflush(None); print(n)")
    r = _run_child(code, path)
    assert r.returncode == 0
    assert r.stdout.decode().splitlines() == ["x=42", "5"]


def test_platform_queries(lib):
    L, _ = lib
    assert L.dwt_util_version()
    assert L.dwt_util_arch().decode() == os.uname().machine
    with open("/proc/sys/kernel/hostname") as f:
        assert L.dwt_util_node().decode() == f.read().strip()
    with open("/proc/self/cmdline", "rb") as f:
        argv0 = f.read().split(b"\0")[0]
    assert L.dwt_util_appname() == os.path.basename(argv0)
    for t in range(13):
        assert L.dwt_util_clock_available(t) == 0
    assert L.dwt_util_clock_available(13) == -1 and L.dwt_util_clock_available(14) == -1
    assert L.dwt_util_get_max_workers() == 1 and L.dwt_util_get_thread_num() == 0
    L.dwt_util_set_num_workers(4)
    L.dwt_util_switch_op(1)


def test_wait_blocks_for_the_interval(lib):
    import time
    L, _ = lib
    t0 = time.perf_counter()
    L.dwt_util_wait(30)
    assert time.perf_counter() - t0 >= 0.029


def test_failed_precondition_logs_and_aborts(lib):
    _, path = lib
    code = "import ctypes as C, sys; L = C.CDLL(sys.argv[1]); L.dwt_zero_padding_i_s(None, 1, 2)"
    r = _run_child(code, path)
    assert r.returncode != 0
    assert b"dwt_zero_padding_i_s: precondition failed" in r.stderr


def test_self_test_without_a_device(lib):
    _, path = lib
    code = "import ctypes as C, sys; L = C.CDLL(sys.argv[1]); L.dwt_util_test()"
    r = subprocess.run([sys.executable, "-c", code, path], capture_output=True, timeout=300,
                       env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert r.returncode == 0
    err = r.stderr.decode()
    assert "TEST: allocate vector of 4096 floats..." in err
    assert "TEST: no CUDA device" in err


@pytest.mark.gpu
def test_self_test_round_trip_on_the_device(lib):
    _, path = lib
    code = "import ctypes as C, sys; L = C.CDLL(sys.argv[1]); L.dwt_util_test()"
    r = _run_child(code, path)
    assert r.returncode == 0, r.stderr.decode()
    err = r.stderr.decode()
    assert "TEST: GPU round trip of a 64x64 image...\nTEST: ok" in err


@pytest.mark.gpu
def test_zero_padding_on_device_memory(lib):
    import torch
    L, _ = lib
    for g in GOLDEN["zero_padding"][::7]:
        dt = torch.float32 if g["t"] == "s" else torch.float64
        n = len(g["out"])
        buf = torch.arange(1, 1 + n, dtype=dt, device="cuda")
        base = buf.data_ptr()
        es = buf.element_size()
        if g["dir"] == "f":
            getattr(L, f"dwt_zero_padding_f_stride_{g['t']}")(base, base + n // 2 * es, g["N"], g["nl"], g["nh"],
                                                              g["stride"])
        else:
            getattr(L, f"dwt_zero_padding_i_stride_{g['t']}")(base, g["N"], g["nd"], g["stride"])
        assert buf.cpu().tolist() == g["out"]


def _build_c_caller(lib_path, tmp_path):
    src = os.path.join(ROOT, "tests", "c", "drop_in_roundtrip.c")
    exe = str(tmp_path / "drop_in_roundtrip")
    libdir = os.path.dirname(lib_path)
    subprocess.run(["gcc", "-std=c99", "-O1", "-I", os.path.join(ROOT, "include"), src, "-o", exe, "-L", libdir,
                    "-ldwt_gb300", f"-Wl,-rpath,{libdir}", "-Wl,--no-undefined", "-lm"], check=True,
                   capture_output=True)
    return exe


def test_c_caller_builds_against_the_header(lib, tmp_path):
    _, path = lib
    assert os.path.exists(_build_c_caller(path, tmp_path))


@pytest.mark.gpu
@pytest.mark.parametrize("size", [(512, 512), (1023, 769)])
def test_c_caller_round_trip_on_the_device(lib, tmp_path, size):
    _, path = lib
    exe = _build_c_caller(path, tmp_path)
    pgm = str(tmp_path / "view.pgm")
    r = subprocess.run([exe, str(size[0]), str(size[1]), pgm], capture_output=True, timeout=300)
    err = r.stderr.decode()
    assert r.returncode == 0, err
    assert f"cdf97 {size[0]}x{size[1]}" in err and err.count("round trip: ok") == 2
    with open(pgm) as f:
        head = [f.readline().strip() for _ in range(3)]
    assert head == ["P2", f"{size[0]} {size[1]}", "255"]
