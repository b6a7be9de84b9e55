// Lifting along one line as a per-thread recurrence (device code shared by
// the coarse-level kernel, the batched kernel's tail items and the signal
// bank kernel).
//
// A thread walks a line two samples at a time, carrying the partial lifting
// results of the previous pairs in registers, and emits output pair p once
// the last lifting step has reached it (LAT = NS/2 pairs later).  Samples
// outside the line are read at their whole-sample symmetric mirror, which
// yields the same values as the reference's boundary handling, sample for
// sample (x + c*(l + r) with l and r swapped).  A line can be cut into
// segments: a segment starts LAT pairs early from zero state, and by the
// time it reaches its first output pair every partial result depends only
// on real samples, so segments are independent and bit-identical to one
// walk over the whole line.
//
// Threads are mapped to consecutive lines, so that in a row-major buffer
// with an odd pitch both the row passes (lanes on rows, stride = pitch) and
// the column passes (lanes on adjacent columns) hit 32 distinct banks.
#pragma once

#include "dwt_common.cuh"

namespace dwt {
namespace recur {

// Lifting state carried between pairs, and one step of it: pair m's raw
// samples in, output pair m - LAT out.
template <int NS>
struct FwdState {
    float e = 0, o = 0, o1 = 0, e1 = 0, o2 = 0;
    __device__ __forceinline__ void step(float A, float B, float &L, float &H, const Wavelet &W)
    {
        if (NS == 4) {
            const float o1n = lift(o, W.c[0], e, A);
            const float e1n = lift(e, W.c[1], o1, o1n);
            const float o2n = lift(o1, W.c[2], e1, e1n);
            const float e2n = lift(e1, W.c[3], o2, o2n);
            L = fmul(e2n, W.zeta_e);
            H = fmul(o2n, W.zeta_o);
            o1 = o1n; e1 = e1n; o2 = o2n;
        } else {
            const float o1n = lift(o, W.c[0], e, A);
            const float e1n = lift(e, W.c[1], o1, o1n);
            L = fmul(e1n, W.zeta_e);
            H = fmul(o1n, W.zeta_o);
            o1 = o1n;
        }
        e = A;
        o = B;
    }
};

template <int NS>
struct InvState {
    float o = 0, e1 = 0, o1 = 0, e2 = 0;
    // Lc, Hc: the coefficient pair m (unscaled); Ev, Ov: samples 2(m-LAT), 2(m-LAT)+1
    __device__ __forceinline__ void step(float Lc, float Hc, float &Ev, float &Ov, const Wavelet &W)
    {
        const float E = fmul(Lc, W.zeta_o);
        const float O = fmul(Hc, W.zeta_e);
        if (NS == 4) {
            const float e1n = lift(E, W.c[0], o, O);
            const float o1n = lift(o, W.c[1], e1, e1n);
            const float e2n = lift(e1, W.c[2], o1, o1n);
            const float o2n = lift(o1, W.c[3], e2, e2n);
            Ev = e2;
            Ov = o2n;
            e1 = e1n; o1 = o1n; e2 = e2n;
        } else {
            const float e1n = lift(E, W.c[0], o, O);
            const float o1n = lift(o, W.c[1], e1, e1n);
            Ev = e1;
            Ov = o1n;
            e1 = e1n;
        }
        o = O;
    }
};

// Forward: samples x[i*xs], i < n (n >= 2); writes L_p to y[p*ys] and H_p to
// y[(nl + p)*ys], nl = ceil(n/2), for output pairs p in [k0, k1).  Pairs
// 0 <= m < n/2 lie inside the line and take the fast path (no mirroring, no
// bound on H); the others read mirrored samples.
template <int NS>
__device__ __forceinline__ void line_forward(const float *x, int xs, int n, float *y, int ys, int k0, int k1,
                                             const Wavelet &W)
{
    constexpr int LAT = NS / 2;
    const int nl = (n + 1) >> 1, mid = n >> 1;
    const int m_end = k1 + LAT;
    FwdState<NS> S;
    auto edge = [&](int m) {
        const int ra = mirror(2 * m, n), rb = mirror(2 * m + 1, n);
        float L, H;
        S.step(x[ra * xs], x[rb * xs], L, H, W);
        const int p = m - LAT;
        if (p >= k0) {
            y[p * ys] = L;
            if (2 * p + 1 < n) y[(nl + p) * ys] = H;
        }
    };
    int m = k0 - LAT;
    for (; m < 0 && m < m_end; ++m) edge(m);
    // interior: the warm-up pairs, then pairs with outputs
    const int body_end = min(m_end, mid);
    const float *xp = x + 2 * m * xs;
    for (; m < body_end && m < k0 + LAT; ++m, xp += 2 * xs) {
        float L, H;
        S.step(xp[0], xp[xs], L, H, W);
    }
    float *yl = y + (m - LAT) * ys, *yh = y + (nl + m - LAT) * ys;
#pragma unroll 2
    for (; m < body_end; ++m, xp += 2 * xs, yl += ys, yh += ys) {
        float L, H;
        S.step(xp[0], xp[xs], L, H, W);
        *yl = L;
        *yh = H;
    }
    for (; m < m_end; ++m) edge(m);
}

// Inverse: L_j at x[j*xs] (j < nl) and H_j at x[(nl + j)*xs]; writes the
// rebuilt samples 2p and 2p+1 to y[(2p)*ys], y[(2p+1)*ys] for p in [k0, k1).
template <int NS>
__device__ __forceinline__ void line_inverse(const float *x, int xs, int n, float *y, int ys, int k0, int k1,
                                             const Wavelet &W)
{
    constexpr int LAT = NS / 2;
    const int nl = (n + 1) >> 1, mid = n >> 1;
    const int m_end = k1 + LAT;
    InvState<NS> S;
    auto edge = [&](int m) {
        const int ra = mirror(2 * m, n), rb = mirror(2 * m + 1, n);
        float Ev, Ov;
        S.step(x[(ra >> 1) * xs], x[(nl + (rb >> 1)) * xs], Ev, Ov, W);
        const int p = m - LAT;
        if (p >= k0) {
            y[(2 * p) * ys] = Ev;
            if (2 * p + 1 < n) y[(2 * p + 1) * ys] = Ov;
        }
    };
    int m = k0 - LAT;
    for (; m < 0 && m < m_end; ++m) edge(m);
    const int body_end = min(m_end, mid);
    const float *lp = x + m * xs, *hp = x + (nl + m) * xs;
    for (; m < body_end && m < k0 + LAT; ++m, lp += xs, hp += xs) {
        float Ev, Ov;
        S.step(*lp, *hp, Ev, Ov, W);
    }
    float *yp = y + 2 * (m - LAT) * ys;
#pragma unroll 2
    for (; m < body_end; ++m, lp += xs, hp += xs, yp += 2 * ys) {
        float Ev, Ov;
        S.step(*lp, *hp, Ev, Ov, W);
        yp[0] = Ev;
        yp[ys] = Ov;
    }
    for (; m < m_end; ++m) edge(m);
}

// Band lines are short (a band that fits one CTA's shared memory), so a
// line segment is lifted as a window held in one thread's registers rather
// than walked: the thread loads its SEG output pairs plus a halo of NS
// samples on each side (mirrored past the ends of the line), applies the NS
// lifting steps uniformly over the whole window, fully unrolled, and stores
// the middle.  Each step leaves one more sample at each end of the window
// stale (it lacks an outer neighbour), and NS steps reach no further than
// NS samples in, so the stored samples are exact.  Mirrored samples lift to
// the mirror images of the lifted samples (x + c*(l + r), l and r swapped),
// so windows at the ends of the line are exact too.
constexpr int kSegPairs = 8;

// Index of window sample r (r >= -NS) of a line of n > NS samples: one
// reflection at each end is exact for every sample an output depends on
// (r <= n - 1 + NS); samples beyond that only feed stale window ends, and
// are clamped to a valid index.
template <int NS>
__device__ __forceinline__ int reflect(int r, int n)
{
    r = abs(r);
    if (r >= n) r = max(2 * (n - 1) - r, 0);
    return r;
}

// hoff: sample index of H_0 in y (ceil(n/2) in the reference layout; the
// outer midpoint in a zero-padded sparse frame).
template <int NS, int SEG>
__device__ __forceinline__ void window_forward(const float *x, int xs, int n, float *y, int ys, int k0,
                                               const Wavelet &W, int hoff)
{
    constexpr int WN = 2 * SEG + 2 * NS;
    const int s0 = 2 * k0 - NS;  // even: window index parity = sample parity
    float v[WN];
    if (s0 >= 0 && s0 + WN <= n) {
#pragma unroll
        for (int i = 0; i < WN; ++i) v[i] = x[(s0 + i) * xs];
    } else if (n > NS) {
#pragma unroll
        for (int i = 0; i < WN; ++i) v[i] = x[reflect<NS>(s0 + i, n) * xs];
    } else {
#pragma unroll
        for (int i = 0; i < WN; ++i) v[i] = x[mirror(s0 + i, n) * xs];
    }
#pragma unroll
    for (int s = 0; s < NS; s += 2) {
#pragma unroll
        for (int i = 1; i < WN - 1; i += 2) v[i] = lift(v[i], W.c[s], v[i - 1], v[i + 1]);
#pragma unroll
        for (int i = 2; i < WN - 1; i += 2) v[i] = lift(v[i], W.c[s + 1], v[i - 1], v[i + 1]);
    }
    const int nl = (n + 1) >> 1;
#pragma unroll
    for (int j = 0; j < SEG; ++j) {
        const int p = k0 + j;
        if (p < nl) {
            y[p * ys] = fmul(v[NS + 2 * j], W.zeta_e);
            if (2 * p + 1 < n) y[(hoff + p) * ys] = fmul(v[NS + 2 * j + 1], W.zeta_o);
        }
    }
}

// Inverse: sample i of the line is L_{i/2} (even i) or H_{i/2} (odd i) with
// its scaling undone; the window holds samples 2*k0 - NS ... and the steps
// run in the inverse order (even samples first).
template <int NS, int SEG>
__device__ __forceinline__ void window_inverse(const float *x, int xs, int n, float *y, int ys, int k0,
                                               const Wavelet &W, int hoff)
{
    constexpr int WN = 2 * SEG + 2 * NS;
    const int nl = hoff;  // H_j at x[(hoff + j) * xs]
    const int s0 = 2 * k0 - NS;
    float v[WN];
    if (s0 >= 0 && s0 + WN <= n) {
        const int j0 = s0 >> 1;
#pragma unroll
        for (int j = 0; j < WN / 2; ++j) {
            v[2 * j] = fmul(x[(j0 + j) * xs], W.zeta_o);
            v[2 * j + 1] = fmul(x[(nl + j0 + j) * xs], W.zeta_e);
        }
    } else {
#pragma unroll
        for (int i = 0; i < WN; ++i) {
            const int r = n > NS ? reflect<NS>(s0 + i, n) : mirror(s0 + i, n);
            v[i] = (r & 1) ? fmul(x[(nl + (r >> 1)) * xs], W.zeta_e) : fmul(x[(r >> 1) * xs], W.zeta_o);
        }
    }
#pragma unroll
    for (int s = 0; s < NS; s += 2) {
#pragma unroll
        for (int i = 2; i < WN - 1; i += 2) v[i] = lift(v[i], W.c[s], v[i - 1], v[i + 1]);
#pragma unroll
        for (int i = 1; i < WN - 1; i += 2) v[i] = lift(v[i], W.c[s + 1], v[i - 1], v[i + 1]);
    }
#pragma unroll
    for (int j = 0; j < SEG; ++j) {
        const int p = k0 + j;
        if (2 * p < n) {
            y[(2 * p) * ys] = v[NS + 2 * j];
            if (2 * p + 1 < n) y[(2 * p + 1) * ys] = v[NS + 2 * j + 1];
        }
    }
}

// One pass over `nl` lines of length n, line l at src + l*ls (sample stride
// xs) into dst + l*ds (stride ys), H at sample hoff (ceil(n/2) by default),
// by threads tid of nthreads, one window
// (line, segment of SEG output pairs) per item; consecutive threads take
// consecutive lines.  Long windows do less halo work, short ones have
// shorter dependency chains per thread.  A line of length 1 is only scaled
// (the reference's one-sample transform).
template <int NS, bool INV, int SEG = kSegPairs>
__device__ __forceinline__ void pass(const float *src, int ls, int xs, float *dst, int ds, int ys, int nl, int n,
                                     const Wavelet &W, int tid, int nthreads, int hoff = -1)
{
    if (hoff < 0) hoff = (n + 1) >> 1;
    if (n == 1) {
        const float z = INV ? W.n1_inv : W.n1_fwd;
        for (int l = tid; l < nl; l += nthreads) dst[l * ds] = fmul(src[l * ls], z);
        return;
    }
    const int nsegs = ((n + 1) / 2 + SEG - 1) / SEG;
    const int items = nl * nsegs;
    for (int t = tid; t < items; t += nthreads) {
        const int sgi = t / nl, l = t - sgi * nl;
        if (INV)
            window_inverse<NS, SEG>(src + l * ls, xs, n, dst + l * ds, ys, sgi * SEG, W, hoff);
        else
            window_forward<NS, SEG>(src + l * ls, xs, n, dst + l * ds, ys, sgi * SEG, W, hoff);
    }
}

// Row-major band buffers with an odd pitch (conflict-free row and column
// passes); two of them hold a band and its half-transformed copy.
__host__ __device__ inline int band_pitch(int w) { return w | 1; }
__host__ __device__ inline long long band_floats(int w, int h) { return 2LL * band_pitch(w) * h; }

// Thread tid's share of the flat indices tid, tid + nthreads, ... of a
// (x1-x0) x (y1-y0) rectangle, visited as (x, y) without a division per
// element.
template <typename F>
__device__ __forceinline__ void for_rect(int x0, int x1, int y0, int y1, int tid, int nthreads, F f)
{
    const int w = x1 - x0;
    if (w <= 0 || y1 <= y0) return;
    int y = tid / w, x = tid - y * w;
    const int dy = nthreads / w, dx = nthreads - dy * w;
    for (y += y0; y < y1;) {
        f(x0 + x, y);
        x += dx;
        y += dy;
        if (x >= w) {
            x -= w;
            ++y;
        }
    }
}

// src[y*sp + x] -> dst[y*dp + x] over [x0,x1) x [y0,y1).
__device__ __forceinline__ void copy_rect(const float *src, long long sp, float *dst, long long dp, int x0, int x1,
                                          int y0, int y1, int tid, int nthreads)
{
    for_rect(x0, x1, y0, y1, tid, nthreads, [&](int x, int y) { dst[y * dp + x] = src[y * sp + x]; });
}

// All `levels` forward levels of the w0 x h0 band held in A (pitch P =
// band_pitch(w0)), B as scratch: rows then columns per level (the
// reference's order); after each level its three detail bands are copied to
// `out` and the LL band stays in the top-left of A.  Ends with the final LL
// copied to `out`.  `sync` is the barrier of the participating threads.
template <int NS, int SEG = kSegPairs, typename Sync>
__device__ __forceinline__ void band_forward(float *A, float *B, int w0, int h0, int levels, float *out,
                                             long long out_pitch, const Wavelet &W, int tid, int nthreads,
                                             Sync sync)
{
    const int P = band_pitch(w0);
    int w = w0, h = h0;
    for (int lvl = 0; lvl < levels; ++lvl) {
        const int wd = (w + 1) >> 1, hd = (h + 1) >> 1;
        pass<NS, false, SEG>(A, P, 1, B, P, 1, h, w, W, tid, nthreads);  // rows
        sync();
        pass<NS, false, SEG>(B, 1, P, A, 1, P, w, h, W, tid, nthreads);  // columns
        sync();
        // detail bands: the w x h region outside [0,hd) x [0,wd)
        copy_rect(A, P, out, out_pitch, wd, w, 0, hd, tid, nthreads);
        copy_rect(A, P, out, out_pitch, 0, w, hd, h, tid, nthreads);
        w = wd;
        h = hd;
    }
    copy_rect(A, P, out, out_pitch, 0, w, 0, h, tid, nthreads);
}

// All `levels` inverse levels of the coefficient region held in A (the
// w0 x h0 top-left of a frame in the reference layout): per level, from the
// coarsest, rows then columns; the rebuilt band ends in A.
template <int NS, int SEG = kSegPairs, typename Sync>
__device__ __forceinline__ void band_inverse(float *A, float *B, int w0, int h0, int levels, const Wavelet &W,
                                             int tid, int nthreads, Sync sync)
{
    const int P = band_pitch(w0);
    for (int lvl = levels - 1; lvl >= 0; --lvl) {
        int w = w0, h = h0;
        for (int k = 0; k < lvl; ++k) {
            w = (w + 1) >> 1;
            h = (h + 1) >> 1;
        }
        pass<NS, true, SEG>(A, P, 1, B, P, 1, h, w, W, tid, nthreads);  // rows
        sync();
        pass<NS, true, SEG>(B, 1, P, A, 1, P, w, h, W, tid, nthreads);  // columns
        sync();
    }
}

}  // namespace recur
}  // namespace dwt
