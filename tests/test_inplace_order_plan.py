"""Host-side check of the ordered in-place level 0 (inplace_device in
libdwt_gb300/csrc/dwt_capi.cu, the drop-in 2D calls on device frames): its
units take tickets in segment order -- bottom-up in the forward, top-down in
the inverse -- and before a unit writes into the caller's frame it waits for
the segments the library names (inplace_readers), which must all come earlier
in that order; segments from stage_seg on go through the staging frame.

The plan comes from the library itself (dwt_gpu_inplace_plan, host code, no
device work) and is checked against the exact rows the level kernel touches,
replayed here: every pair a unit walks (its segment warmed up by the lifting
latency on both sides, rounded up to whole two-pair stages), the mirrored rows
at the borders, the LH / HH rows written (forward) or read (inverse).  For
every pair of segments where one writes a frame row the other reads, the
reader must be in the writer's wait range and come earlier in the order, or
read / write that row in the staging frame."""
import ctypes as C
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEIGHTS = [2, 3, 5, 33, 100, 257, 1024, 1025, 2047, 2048, 4099, 8192, 16383, 16384, 16385]


def _lib():
    from libdwt_gb300.buildext import build
    lib = C.CDLL(build())
    f = lib.dwt_gpu_inplace_plan
    f.argtypes = [C.c_int] * 5 + [C.POINTER(C.c_int)] * 3 + [C.c_void_p]
    f.restype = C.c_int
    return lib


def plan(lib, wavelet, inverse, w, h, dy=-1):
    S, n, st = C.c_int(), C.c_int(), C.c_int()
    assert lib.dwt_gpu_inplace_plan(wavelet, inverse, w, h, dy, C.byref(S), C.byref(n), C.byref(st), None) == 0
    rng = (C.c_int * (2 * n.value))()
    assert lib.dwt_gpu_inplace_plan(wavelet, inverse, w, h, dy, C.byref(S), C.byref(n), C.byref(st), rng) == 0
    return S.value, n.value, st.value, [(rng[2 * s], rng[2 * s + 1]) for s in range(n.value)]


def mirror(r, n):
    p = 2 * (n - 1)
    m = r % p
    return p - m if m >= n else m


def pair_rows(m, h):
    ra, rb = 2 * m, 2 * m + 1
    if ra < 0 or rb >= h:
        ra, rb = mirror(2 * m, h), mirror(2 * m + 1, h)
    return ra, rb


def walked_pairs(s, S, h, lat):
    npairs = (h + 1) // 2
    k0 = s * S
    k1 = min(k0 + S, npairs)
    total = k1 - k0 + 2 * lat
    iters = (total + 1) // 2
    return range(k0 - lat, k0 - lat + 2 * iters), range(k0, k1)


def check(lib, wavelet, inverse, h, w=4096, dy=None):
    """dy: frame row of the LH / HH bands (the outer midpoint of a sparse
    frame; (h + 1) // 2 for a dense one)."""
    lat = 2 if wavelet == 0 else 1
    hs = (h + 1) // 2 if dy is None else dy
    S, n, st, rng = plan(lib, wavelet, inverse, w, h, -1 if dy is None else dy)
    reads, writes = [], []
    for s in range(n):
        walk, out = walked_pairs(s, S, h, lat)
        if not inverse:
            rr = set()
            for m in walk:
                rr.update(pair_rows(m, h))
            ww = {hs + p for p in out if p <= h // 2 - 1}
        else:
            rr = {hs + (pair_rows(m, h)[1] >> 1) for m in walk}
            ww = set()
            for p in out:
                ww.add(2 * p)
                if p <= h // 2 - 1:
                    ww.add(2 * p + 1)
        reads.append(rr)
        writes.append(ww)
    top = hs + h // 2  # end of the LH / HH rows
    if not inverse:
        staged_lo = hs + st * S if st < n else top
        for s in range(n):
            if s >= st:
                assert all(r >= staged_lo for r in writes[s]), (h, s)
                continue
            a, b = rng[s]
            for r in range(n):
                if writes[s] & reads[r]:
                    # r reads rows s overwrites: s waits for r, which runs first
                    assert a <= r <= b and r > s, (h, s, r, rng[s])
    else:
        staged_lo = min(top, max(hs, hs + max(0, st * S - lat - 3))) if st < n else top
        for r in range(st, n):
            assert all(x >= staged_lo for x in reads[r]), (h, r)
        for wr in range(n):
            a, b = rng[wr]
            for r in range(min(st, n)):
                if writes[wr] & reads[r]:
                    assert a <= r <= b and r < wr, (h, wr, r, rng[wr])
    return S, n, st


@pytest.mark.parametrize("wavelet", [0, 1])
@pytest.mark.parametrize("inverse", [0, 1])
@pytest.mark.parametrize("h", HEIGHTS)
def test_ordered_plan_covers_every_hazard(wavelet, inverse, h):
    S, n, st = check(_lib(), wavelet, inverse, h)
    # only the segments at the end of the order pass through T
    assert n - st <= 2 * 16 + 8, (S, n, st)  # default lead: 16 segments


def test_ordered_plan_with_other_leads():
    """The plan with no lead and with a long one (DWT_GPU_INPLACE_LEAD is read
    once per process: child processes)."""
    code = ("import sys; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
            "import test_inplace_order_plan as T\n"
            "lib = T._lib()\n"
            "for wv in (0, 1):\n"
            "    for inv in (0, 1):\n"
            "        for h in T.HEIGHTS:\n"
            "            T.check(lib, wv, inv, h)\n"
            "print('plans ok')\n") % (ROOT, os.path.join(ROOT, "tests"))
    for lead in ("0", "1", "40"):
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600,
                           env=dict(os.environ, DWT_GPU_INPLACE_LEAD=lead))
        assert r.returncode == 0 and "plans ok" in r.stdout, r.stdout + r.stderr


@pytest.mark.parametrize("wavelet", [0, 1])
@pytest.mark.parametrize("inverse", [0, 1])
@pytest.mark.parametrize("h,dy", [(12000, 8192), (1000, 1024), (1025, 513), (3001, 2048), (700, 4096)])
def test_ordered_plan_sparse_frames(wavelet, inverse, h, dy):
    """An inner image in a larger zero-padded frame: the LH / HH bands start
    at the outer midpoint, below the inner image's own midpoint."""
    check(_lib(), wavelet, inverse, h, dy=dy)


def test_plan_refuses_bad_arguments():
    lib = _lib()
    S, n, st = C.c_int(), C.c_int(), C.c_int()
    assert lib.dwt_gpu_inplace_plan(0, 0, 1, 1024, -1, C.byref(S), C.byref(n), C.byref(st), None) == -1
    assert lib.dwt_gpu_inplace_plan(7, 0, 1024, 1024, -1, C.byref(S), C.byref(n), C.byref(st), None) == -1
    assert lib.dwt_gpu_inplace_plan(0, 0, 1024, 1024, 511, C.byref(S), C.byref(n), C.byref(st), None) == -1
