"""CPU check of the decomposition the fused sparse-frame path runs on the GPU
(sparse_inplace in libdwt_gb300/csrc/dwt_capi.cu): for an outer frame with
an inner image and zero padding, the reference's in-place level sequence
(src/libdwt.c:6330-6397 forward, 6677-6745 inverse) equals

  forward: for the fused levels, one dense level of the inner LL band with
           its H bands placed at the OUTER midpoints; the reference's own
           per-line sequence for the remaining small levels on the top-left
           sub-frame; then zeros in the rectangles of each fused level's
           frame that none of its bands (nor the next level's frame) covers;
  inverse: the per-line sequence for the small levels first, then dense
           inverse levels reading the H bands at the outer midpoints; then
           zeros outside the inner image.

Both sides are computed by the oracle (bit-exact with the reference), the
composition by the same steps and the same zero rectangles as the GPU code,
over random geometries, both wavelets.  The final forward layout is also
checked against a per-sample band predicate: a band of some level, or zero."""
import numpy as np
import pytest

from oracle import oracle as O


def cdp(v, j):
    return -(-v // (1 << j))


def fast(iw, ih):
    return iw >= 16 and ih >= 16 and iw * ih > 4096


def covered(x, y, ox, oy, ix, iy, J):
    """Whether a sample holds a band of some level (final layout)."""
    for j in range(J):
        odx, ody = cdp(ox, j + 1), cdp(oy, j + 1)
        iw, ih = cdp(ix, j), cdp(iy, j)
        if x < odx and y < ody:
            if j == J - 1:
                return x < (iw + 1) // 2 and y < (ih + 1) // 2
            continue
        in_x = x < (iw + 1) // 2 or (odx <= x < odx + iw // 2)
        in_y = y < (ih + 1) // 2 or (ody <= y < ody + ih // 2)
        return in_x and in_y
    return False


def band_mask(ox, oy, ix, iy, J):
    m = np.zeros((oy, ox), bool)
    for y in range(oy):
        for x in range(ox):
            m[y, x] = covered(x, y, ox, oy, ix, iy, J)
    return m


def zero_rects(jf, J, ox, oy, ix, iy):
    """The rectangles sparse_inplace zeroes after the fused forward levels
    (x0, y0, w, h), as the GPU code lists them."""
    rects = []
    for j in range(jf):
        ow, oh, dx, dy = cdp(ox, j), cdp(oy, j), cdp(ox, j + 1), cdp(oy, j + 1)
        iw, ih = cdp(ix, j), cdp(iy, j)
        lx, hx, ly, hy = (iw + 1) // 2, iw // 2, (ih + 1) // 2, ih // 2
        rects += [(lx, dy, dx - lx, oh - dy), (dx + hx, 0, ow - dx - hx, oh), (dx, ly, hx, dy - ly),
                  (0, dy + hy, lx, oh - dy - hy), (dx, dy + hy, hx, oh - dy - hy)]
        if j == J - 1:
            rects += [(lx, 0, dx - lx, dy), (0, ly, lx, dy - ly)]
    return [r for r in rects if r[2] > 0 and r[3] > 0]


def reference(frame, wav, direction, ox, oy, ix, iy, J):
    a = frame.copy()
    O.transform2(a.view(np.uint8).reshape(-1), wav, direction, ox * 4, 4, (ox, oy), (ix, iy), J, 0, 1)
    return a


def sub_frame_levels(frame, wav, direction, ox, oy, ix, iy, j0, J):
    """The reference's per-line levels j0 .. J-1 (forward) or J .. j0+1
    (inverse) on the top-left sub-frame, through the reference driver run on
    that sub-frame (level geometry composes: cdp(cdp(o, j0), k) = cdp(o, j0 + k))."""
    sx, sy = cdp(ox, j0), cdp(oy, j0)
    sub = np.ascontiguousarray(frame[:sy, :sx]).copy()
    O.transform2(sub.view(np.uint8).reshape(-1), wav, direction, sx * 4, 4, (sx, sy), (cdp(ix, j0), cdp(iy, j0)),
                 J - j0, 0, 1)
    frame[:sy, :sx] = sub


def composed_forward(frame, wav, ox, oy, ix, iy, J):
    out = frame.copy()
    jf = 0
    while jf < J and fast(cdp(ix, jf), cdp(iy, jf)):
        jf += 1
    ll = frame[:iy, :ix].copy()
    for j in range(jf):
        iw, ih = cdp(ix, j), cdp(iy, j)
        dx, dy = cdp(ox, j + 1), cdp(oy, j + 1)
        d, _ = O.transform2_dense(ll, wav, "f", 1)
        lx, ly = (iw + 1) // 2, (ih + 1) // 2
        out[:ly, dx:dx + iw // 2] = d[:ly, lx:]
        out[dy:dy + ih // 2, :lx] = d[ly:, :lx]
        out[dy:dy + ih // 2, dx:dx + iw // 2] = d[ly:, lx:]
        ll = d[:ly, :lx].copy()
    out[:ll.shape[0], :ll.shape[1]] = ll
    if jf < J:
        sub_frame_levels(out, wav, "f", ox, oy, ix, iy, jf, J)
    for (x0, y0, w, h) in zero_rects(jf, J, ox, oy, ix, iy):
        out[y0:y0 + h, x0:x0 + w] = 0.0
    return out, jf


def composed_inverse(frame, wav, ox, oy, ix, iy, J):
    out = frame.copy()
    jf = 0
    while jf < J and fast(cdp(ix, jf), cdp(iy, jf)):
        jf += 1
    if jf < J:
        sub_frame_levels(out, wav, "i", ox, oy, ix, iy, jf, J)
    details = frame.copy()  # the staged level-0 details (T): untouched input
    ll = out[:cdp(iy, jf), :cdp(ix, jf)].copy()
    for j in range(jf, 0, -1):
        iw, ih = cdp(ix, j - 1), cdp(iy, j - 1)
        src = details if j == 1 else out
        sx, sy = cdp(ox, j), cdp(oy, j)
        lx, ly = (iw + 1) // 2, (ih + 1) // 2
        d = np.empty((ih, iw), np.float32)
        d[:ly, :lx] = ll
        d[:ly, lx:] = src[:ly, sx:sx + iw // 2]
        d[ly:, :lx] = src[sy:sy + ih // 2, :lx]
        d[ly:, lx:] = src[sy:sy + ih // 2, sx:sx + iw // 2]
        ll, _ = O.transform2_dense(d, wav, "i", 1)
    res = np.zeros_like(out)
    res[:iy, :ix] = ll
    return res, jf


GEOMS = [
    # (ox, oy, ix, iy)
    (128, 128, 100, 90),
    (160, 97, 131, 80),
    (256, 64, 200, 33),
    (96, 200, 70, 170),
    (257, 129, 256, 128),
    (512, 300, 300, 280),
    (512, 512, 20, 400),
    (200, 200, 199, 199),
    (64, 2048, 40, 1500),
]


@pytest.mark.parametrize("wav", ["cdf97", "cdf53"])
@pytest.mark.parametrize("geom", GEOMS)
def test_composition_equals_reference_sequence(wav, geom):
    ox, oy, ix, iy = geom
    rng = np.random.default_rng(ox * 7 + oy * 13 + ix + iy)
    frame = rng.uniform(-50, 300, size=(oy, ox)).astype(np.float32)  # stale samples outside the inner image too
    jl = int(np.ceil(np.log2(min(ox, oy))))
    for J in sorted({1, 2, 3, jl}):
        ref_f = reference(frame, wav, "f", ox, oy, ix, iy, J)
        got_f, jf = composed_forward(frame, wav, ox, oy, ix, iy, J)
        assert jf >= 1
        assert np.array_equal(got_f.view(np.uint32), ref_f.view(np.uint32)), (geom, J, "forward")
        # the final layout: a band or zero everywhere in the outer frame
        assert not ref_f[~band_mask(ox, oy, ix, iy, J)].any()
        # the inverse of arbitrary coefficients (stale samples everywhere else)
        coef = ref_f.copy()
        coef[~band_mask(ox, oy, ix, iy, J)] = rng.uniform(-9, 9, size=int((~band_mask(ox, oy, ix, iy, J)).sum()))
        ref_i = reference(coef, wav, "i", ox, oy, ix, iy, J)
        got_i, _ = composed_inverse(coef, wav, ox, oy, ix, iy, J)
        assert np.array_equal(got_i.view(np.uint32), ref_i.view(np.uint32)), (geom, J, "inverse")
