"""Host-side check of the in-place band plan (inplace_device in
libdwt_gb300/csrc/dwt_capi.cu): level 0 of an in-place transform runs as
row bands in a fixed order, and a band writes (forward) or reads (inverse)
the LH / HH rows in the caller's frame only when the host's row-interval test
says no band reading or writing after it can meet those rows.

This replays the plan (segment planning as plan_level, the bands, the
interval test with its margins) and checks it against the exact rows the
level kernel touches -- every pair a unit walks, with the lifting warm-up
and the mirrored rows at the borders -- for both wavelets, odd and even
heights and several band counts: no in-frame write of a band may meet a row
that the same or a later band reads (forward), and no in-frame read may meet
a row that an earlier or the same band writes (inverse)."""
import math

import pytest


def mirror(r, n):
    if n <= 1:
        return 0
    p = 2 * (n - 1)
    m = r % p
    return p - m if m >= n else m


def pair_rows(m, h):
    ra, rb = 2 * m, 2 * m + 1
    if ra < 0 or rb >= h:
        ra, rb = mirror(2 * m, h), mirror(2 * m + 1, h)
    return ra, rb


def plan(h, inverse):
    """Segment length and count of a 2D level of height h (plan_level)."""
    npairs = (h + 1) // 2
    if not inverse:
        seg = max(math.ceil(npairs / 176), 4 if npairs >= 1024 else 2)
    elif npairs > 1024:
        seg = max(math.ceil(npairs / 384), 16)
    else:
        seg = max(math.ceil(npairs / 128), 2)
    seg = min(seg, max(npairs, 1))
    return seg, math.ceil(npairs / seg)


def band_plan(h, lat, inverse, K_env=8):
    hs = (h + 1) // 2
    npairs = hs
    S, nsegs = plan(h, inverse)
    K = min(K_env, nsegs)

    def segs(k):
        if not inverse:
            return nsegs - (k + 1) * nsegs // K, nsegs - k * nsegs // K
        return k * nsegs // K, (k + 1) * nsegs // K

    pairs = [(a * S, min(npairs, b * S)) for a, b in (segs(k) for k in range(K))]
    margin = 2

    def meets(x, y):
        return x[1] > x[0] and y[1] > y[0] and x[0] < y[1] and y[0] < x[1]

    fwd_reads = lambda q: (max(0, 2 * (q[0] - lat) - margin), min(h, 2 * (q[1] + lat) + margin))
    fwd_det = lambda q: (hs + q[0], min(h, hs + q[1]))
    inv_reads = lambda q: (hs + max(0, q[0] - lat - margin), min(h, hs + q[1] + lat + margin))
    inv_writes = lambda q: (2 * q[0], min(h, 2 * q[1]))
    in_frame = []
    staged_lo = h
    for k in range(K):
        if not inverse:
            w = fwd_det(pairs[k])
            ok = all(not meets(w, fwd_reads(pairs[c])) for c in range(k, K))
            if not ok:
                staged_lo = min(staged_lo, w[0])
        else:
            r = inv_reads(pairs[k])
            ok = all(not meets(inv_writes(pairs[b]), r) for b in range(0, k + 1))
            if not ok:
                staged_lo = min(staged_lo, r[0])
        in_frame.append(ok)
    if not inverse:
        in_frame = [f and fwd_det(pairs[k])[0] < staged_lo for k, f in enumerate(in_frame)]
    return S, nsegs, K, [segs(k) for k in range(K)], in_frame, staged_lo


def unit_pairs(seg, S, npairs, lat):
    k0 = seg * S
    k1 = min(k0 + S, npairs)
    return range(k0 - lat, k1 + lat), range(k0, k1)


@pytest.mark.parametrize("lat", [2, 1])
@pytest.mark.parametrize("h", [1024, 1025, 2047, 2048, 4099, 8192, 16383, 16384, 16385])
@pytest.mark.parametrize("K", [3, 8, 16])
def test_forward_bands_write_only_rows_nobody_reads_later(lat, h, K):
    hs = (h + 1) // 2
    S, nsegs, K, segs, in_frame, staged_lo = band_plan(h, lat, False, K)
    last_h = h // 2 - 1
    reads = []   # exact image rows read by each band
    writes = []  # exact LH / HH frame rows each band writes
    for a, b in segs:
        rr, ww = set(), set()
        for sg in range(a, b):
            walk, out = unit_pairs(sg, S, hs, lat)
            for m in walk:
                rr.update(pair_rows(m, h))
            ww.update(hs + p for p in out if p <= last_h)
        reads.append(rr)
        writes.append(ww)
    for k in range(K):
        if in_frame[k]:
            for c in range(k, K):
                assert not (writes[k] & reads[c]), (h, lat, K, k, c)
            assert not any(r >= staged_lo for r in writes[k])
        else:
            assert all(r >= staged_lo for r in writes[k])
    assert sum(in_frame) >= K - 3


@pytest.mark.parametrize("lat", [2, 1])
@pytest.mark.parametrize("h", [1024, 1025, 2047, 2048, 4099, 8192, 16383, 16384, 16385])
@pytest.mark.parametrize("K", [3, 8, 16])
def test_inverse_bands_read_only_rows_nobody_wrote(lat, h, K):
    hs = (h + 1) // 2
    S, nsegs, K, segs, in_frame, staged_lo = band_plan(h, lat, True, K)
    last_odd = h // 2 - 1
    reads, writes = [], []  # LH / HH frame rows read; image rows written
    for a, b in segs:
        rr, ww = set(), set()
        for sg in range(a, b):
            walk, out = unit_pairs(sg, S, hs, lat)
            for m in walk:
                ra, rb = pair_rows(m, h)
                rr.add(hs + (rb >> 1))
            for p in out:
                ww.add(2 * p)
                if p <= last_odd:
                    ww.add(2 * p + 1)
        reads.append(rr)
        writes.append(ww)
    for k in range(K):
        if in_frame[k]:
            for b in range(0, k + 1):
                assert not (writes[b] & reads[k]), (h, lat, K, k, b)
        else:
            # staged bands read T, which holds every LH / HH row they read
            assert all(r >= staged_lo for r in reads[k])
    assert sum(in_frame) >= K - 3
