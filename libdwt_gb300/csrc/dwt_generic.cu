// Layout and frame kernels around the fused level kernel:
//   * repack / unpack between the caller's byte-strided layout (any byte
//     strides, floats possibly not 4-byte aligned) and a compact row-major
//     float frame with a 16-byte aligned pitch;
//   * the per-line path for sparse frames (outer size > inner size), which
//     must keep the reference's exact in-place semantics: a line pass writes
//     L to [0, ceil(n/2)) and H from the outer midpoint, leaving the samples
//     in between untouched (src/libdwt.c:6354-6375), then optional zero
//     padding (src/libdwt.c:6377-6397, 6729-6745).
#include "dwt_generic.cuh"
#include "dwt_recur.cuh"

#include <algorithm>
#include <cstdint>
#include <cstdlib>

namespace dwt {

namespace {

__device__ __forceinline__ float load_any(const unsigned char *p)
{
    if ((reinterpret_cast<uintptr_t>(p) & 3) == 0) return *reinterpret_cast<const float *>(p);
    uint32_t u = uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
    return __uint_as_float(u);
}

__device__ __forceinline__ void store_any(unsigned char *p, float v)
{
    if ((reinterpret_cast<uintptr_t>(p) & 3) == 0) {
        *reinterpret_cast<float *>(p) = v;
        return;
    }
    const uint32_t u = __float_as_uint(v);
    p[0] = u & 0xff;
    p[1] = (u >> 8) & 0xff;
    p[2] = (u >> 16) & 0xff;
    p[3] = (u >> 24) & 0xff;
}

__global__ void repack_kernel(const unsigned char *src, long long sx, long long sy, int ox, int oy,
                              float *dst, long long dpitch)
{
    const long long n = (long long)ox * oy;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const int y = int(k / ox), x = int(k % ox);
        dst[y * dpitch + x] = load_any(src + y * sx + x * sy);
    }
}

__global__ void unpack_kernel(const float *src, long long spitch, unsigned char *dst, long long sx,
                              long long sy, int ox, int oy)
{
    const long long n = (long long)ox * oy;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const int y = int(k / ox), x = int(k % ox);
        store_any(dst + y * sx + x * sy, src[y * spitch + x]);
    }
}

// Rows of per_row elements of V from src (pitch spitch bytes) to dst (pitch
// dpitch bytes): the copy of the host-frame paths where the GPU addresses the
// caller's host memory itself.  Four independent moves per thread and step
// keep enough bytes in flight over the host link.
template <typename V>
__global__ void copy_rows_kernel(const unsigned char *src, long long spitch, unsigned char *dst, long long dpitch,
                                 int per_row, int rows)
{
    const int step = gridDim.x * blockDim.x;
    for (int r = blockIdx.y; r < rows; r += gridDim.y) {
        const V *sr = reinterpret_cast<const V *>(src + r * spitch);
        V *dr = reinterpret_cast<V *>(dst + r * dpitch);
        int i = blockIdx.x * blockDim.x + threadIdx.x;
        for (; i + 3 * step < per_row; i += 4 * step) {
            const V a = sr[i], b = sr[i + step], c = sr[i + 2 * step], d = sr[i + 3 * step];
            dr[i] = a;
            dr[i + step] = b;
            dr[i + 2 * step] = c;
            dr[i + 3 * step] = d;
        }
        for (; i < per_row; i += step) dr[i] = sr[i];
    }
}

// Strided signal gather/scatter: signal s, sample i lives at byte offset
// (s / group) * group_stride + (s % group) * lane_stride + i * stride.
__global__ void gather_signals_kernel(const unsigned char *base, int N, long long stride, long long count,
                                      int group, long long group_stride, long long lane_stride,
                                      float *dst, long long dpitch)
{
    const long long n = (long long)N * count;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const long long s = k / N;
        const int i = int(k % N);
        const unsigned char *p = base + (s / group) * group_stride + (s % group) * lane_stride + i * stride;
        dst[s * dpitch + i] = load_any(p);
    }
}

__global__ void scatter_signals_kernel(const float *src, long long spitch, int N, unsigned char *base,
                                       long long stride, long long count, int group,
                                       long long group_stride, long long lane_stride)
{
    const long long n = (long long)N * count;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const long long s = k / N;
        const int i = int(k % N);
        unsigned char *p = base + (s / group) * group_stride + (s % group) * lane_stride + i * stride;
        store_any(p, src[s * spitch + i]);
    }
}

// One lifting step on the samples of `parity` of a line held in tmp with
// element stride ts (lines interleaved so threads of a warp coalesce).
__device__ __forceinline__ void line_step(float *x, long long ts, int N, int parity, float c)
{
    for (int i = parity; i < N; i += 2) {
        const float l = (i > 0) ? x[(i - 1) * ts] : x[(i + 1) * ts];
        const float r = (i + 1 < N) ? x[(i + 1) * ts] : x[(i - 1) * ts];
        x[i * ts] = lift(x[i * ts], c, l, r);
    }
}

__device__ __forceinline__ void line_scale(float *x, long long ts, int N, float even, float odd)
{
    for (int i = 0; i < N; i += 2) x[i * ts] = fmul(x[i * ts], even);
    for (int i = 1; i < N; i += 2) x[i * ts] = fmul(x[i * ts], odd);
}

// Forward transform of one line in place: reads N samples (es apart),
// writes L to [0, ceil(N/2)) and H to [hoff, hoff + floor(N/2)); x is the
// line's working copy, ts floats between its samples.
__device__ __forceinline__ void line_forward_one(float *line, long long es, int N, int hoff, float *x, long long ts,
                                                 const Wavelet &W)
{
    if (N <= 0) return;
    if (N == 1) {
        line[0] = fmul(line[0], W.n1_fwd);
        return;
    }
    for (int i = 0; i < N; ++i) x[i * ts] = line[i * es];
    for (int s = 0; s < W.nsteps; ++s) line_step(x, ts, N, (s & 1) ? 0 : 1, W.c[s]);
    line_scale(x, ts, N, W.zeta_e, W.zeta_o);
    for (int i = 0; 2 * i < N; ++i) line[i * es] = x[(2 * i) * ts];
    for (int i = 0; 2 * i + 1 < N; ++i) line[(hoff + i) * es] = x[(2 * i + 1) * ts];
}

// Inverse transform of one line: L from [0, ceil(N/2)), H from [hoff, ...),
// result to [0, N).
__device__ __forceinline__ void line_inverse_one(float *line, long long es, int N, int hoff, float *x, long long ts,
                                                 const Wavelet &W)
{
    if (N <= 0) return;
    if (N == 1) {
        line[0] = fmul(line[0], W.n1_inv);
        return;
    }
    for (int i = 0; 2 * i < N; ++i) x[(2 * i) * ts] = line[i * es];
    for (int i = 0; 2 * i + 1 < N; ++i) x[(2 * i + 1) * ts] = line[(hoff + i) * es];
    line_scale(x, ts, N, W.zeta_o, W.zeta_e);
    for (int s = 0; s < W.nsteps; ++s) line_step(x, ts, N, (s & 1) ? 1 : 0, W.c[s]);
    for (int i = 0; i < N; ++i) line[i * es] = x[i * ts];
}

// Per-line transforms in place on a compact frame: line k starts at
// base + k*ls, samples es apart; one thread per line, the lines' working
// copies interleaved in tmp so the threads of a warp coalesce.
__global__ void lines_forward_kernel(float *base, long long ls, long long es, int nlines, int N,
                                     int hoff, float *tmp, const Wavelet W)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nlines) return;
    line_forward_one(base + k * ls, es, N, hoff, tmp + k, nlines, W);
}

__global__ void lines_inverse_kernel(float *base, long long ls, long long es, int nlines, int N,
                                     int hoff, float *tmp, const Wavelet W)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nlines) return;
    line_inverse_one(base + k * ls, es, N, hoff, tmp + k, nlines, W);
}

// Zero padding of a forward level (dwt_zero_padding_f_stride_s): per line,
// zero L samples [ceil(N/2), nL) and H samples [floor(N/2), nH) from hoff.
__device__ __forceinline__ void zero_forward_one(float *line, long long es, int N, int nL, int nH, int hoff)
{
    for (int i = (N + 1) / 2; i < nL; ++i) line[i * es] = 0.0f;
    for (int i = N / 2; i < nH; ++i) line[(hoff + i) * es] = 0.0f;
}

__global__ void zero_forward_kernel(float *base, long long ls, long long es, int nlines, int N, int nL,
                                    int nH, int hoff)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nlines || (nL == 0 && nH == 0)) return;
    zero_forward_one(base + k * ls, es, N, nL, nH, hoff);
}

// Zero padding of an inverse level (dwt_zero_padding_i_stride_s).
__global__ void zero_inverse_kernel(float *base, long long ls, long long es, int nlines, int N, int n_dst)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nlines) return;
    float *line = base + k * ls;
    for (int i = N; i < n_dst; ++i) line[i * es] = 0.0f;
}

// The small levels of a zero-padded sparse frame in one CTA: the level
// frame of the first of them (fx x fy samples of f, pitch in floats) is
// brought into shared memory and every level runs there as the dense inner
// level with its H bands at the outer midpoints -- a row pass over the inner
// rows, a column pass over the L and H columns, both as per-thread lifting
// windows (dwt_recur.cuh) -- followed by zeros over the rest of the level's
// frame, which is what the reference's per-line sequence with zero padding
// leaves there (src/libdwt.c:6353-6397, 6700-6745; the samples it computes
// outside the inner bands are overwritten or zeroed).  Forward levels j0 ..
// j1-1, inverse levels j1 .. j0+1 (j0 < j1), sizes by ceil_div_pow2 of the
// outer and inner sizes of level 0.
constexpr int kTailThreads = 512;
// windows of 2 output pairs, as in the coarse kernel: these levels are
// latency-bound and short per-thread chains win
constexpr int kTailWindowPairs = 2;

template <int NS, bool INV>
__global__ void __launch_bounds__(kTailThreads) sparse_tail_kernel(float *f, long long pitch, int ox, int oy, int ix,
                                                                   int iy, int j0, int j1, const Wavelet W)
{
    extern __shared__ float sh[];
    const int fx = ceil_div_pow2(ox, j0), fy = ceil_div_pow2(oy, j0);
    const int ps = fx | 1;  // odd pitch: the lines of a column pass fall in different banks
    float *S = sh, *T = sh + ps * fy;
    const int tid = threadIdx.x, nt = blockDim.x;
    recur::for_rect(0, fx, 0, fy, tid, nt, [&](int x, int y) { S[y * ps + x] = f[(long long)y * pitch + x]; });
    __syncthreads();
    // zeros over [0, w) x [0, h) of S outside the rectangles [x0, x1) x [y0, y1) of `keep`
    auto zero_outside = [&](int w, int h, const int (*keep)[4], int nk) {
        recur::for_rect(0, w, 0, h, tid, nt, [&](int x, int y) {
            for (int k = 0; k < nk; ++k)
                if (x >= keep[k][0] && x < keep[k][1] && y >= keep[k][2] && y < keep[k][3]) return;
            S[y * ps + x] = 0.0f;
        });
    };
    for (int step = 0; step < j1 - j0; ++step) {
        if (!INV) {
            const int j = j0 + step;
            const int osx = ceil_div_pow2(ox, j), osy = ceil_div_pow2(oy, j);
            const int odx = ceil_div_pow2(ox, j + 1), ody = ceil_div_pow2(oy, j + 1);
            const int isx = ceil_div_pow2(ix, j), isy = ceil_div_pow2(iy, j);
            const int lx = (isx + 1) / 2, hx = isx / 2, ly = (isy + 1) / 2, hy = isy / 2;
            recur::pass<NS, false, kTailWindowPairs>(S, ps, 1, T, ps, 1, isy, isx, W, tid, nt, odx);  // inner rows
            __syncthreads();
            recur::pass<NS, false, kTailWindowPairs>(T, 1, ps, S, 1, ps, lx, isy, W, tid, nt, ody);  // L columns
            recur::pass<NS, false, kTailWindowPairs>(T + odx, 1, ps, S + odx, 1, ps, hx, isy, W, tid, nt, ody);  // H columns
            __syncthreads();
            const int keep[4][4] = {{0, lx, 0, ly}, {odx, odx + hx, 0, ly}, {0, lx, ody, ody + hy},
                                    {odx, odx + hx, ody, ody + hy}};
            zero_outside(osx, osy, keep, 4);
            __syncthreads();
        } else {
            const int j = j1 - step;  // LL_j -> LL_{j-1}
            const int osx = ceil_div_pow2(ox, j), osy = ceil_div_pow2(oy, j);
            const int odx = ceil_div_pow2(ox, j - 1), ody = ceil_div_pow2(oy, j - 1);
            const int idx = ceil_div_pow2(ix, j - 1), idy = ceil_div_pow2(iy, j - 1);
            const int ly = (idy + 1) / 2, hy = idy / 2;
            // rows holding bands (L rows at the top, H rows from the outer midpoint)
            recur::pass<NS, true, kTailWindowPairs>(S, ps, 1, T, ps, 1, ly, idx, W, tid, nt, osx);
            recur::pass<NS, true, kTailWindowPairs>(S + osy * ps, ps, 1, T + osy * ps, ps, 1, hy, idx, W, tid, nt, osx);
            __syncthreads();
            recur::pass<NS, true, kTailWindowPairs>(T, 1, ps, S, 1, ps, idx, idy, W, tid, nt, osy);
            __syncthreads();
            const int keep[1][4] = {{0, idx, 0, idy}};
            zero_outside(odx, ody, keep, 1);
            __syncthreads();
        }
    }
    recur::for_rect(0, fx, 0, fy, tid, nt, [&](int x, int y) { f[(long long)y * pitch + x] = S[y * ps + x]; });
}

// Zero fill of a list of rectangles of a frame (pitch in floats): blocks take
// the rectangles' rows in turn, their threads the row's samples.
__global__ void zero_rects_kernel(float *f, long long pitch, const ZeroRects R)
{
    for (int r = blockIdx.x; r < R.total_rows; r += gridDim.x) {
        int k = 0;
        while (k + 1 < R.n && R.first_row[k + 1] <= r) ++k;
        const int y = R.y0[k] + (r - R.first_row[k]);
        float *row = f + (long long)y * pitch + R.x0[k];
        const int w = R.w[k];
        if ((reinterpret_cast<uintptr_t>(row) & 15) == 0 && (w & 3) == 0) {
            float4 *row4 = reinterpret_cast<float4 *>(row);
            for (int x = threadIdx.x; x < (w >> 2); x += blockDim.x) row4[x] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            for (int x = threadIdx.x; x < w; x += blockDim.x) row[x] = 0.0f;
        }
    }
}

// Signals of separate calls gathered into the rows of a compact frame and
// scattered back: call k's samples i live at a[k] + i * stride[k] bytes
// (forward: N samples; inverse: ceil(N/2) of L at a[k] into [0, ..) and
// floor(N/2) of H at b[k] into [h_off, ..)); results go to c[k] (forward: L
// and then H to h[k]; inverse: N samples), same strides.
__global__ void gather_calls_kernel(const CallRow *calls, const __grid_constant__ CallRowsParam P, int n_calls, int N,
                                    bool inverse, float *dst, long long dpitch, int h_off)
{
    const int k = blockIdx.y;
    if (k >= n_calls) return;
    const CallRow r = calls ? calls[k] : P.r[k];
    float *row = dst + (long long)k * dpitch;
    const int nl = (N + 1) / 2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        if (!inverse || i < nl)
            row[i] = load_any(static_cast<const unsigned char *>(r.a) + (long long)i * r.stride);
        else
            row[h_off + (i - nl)] = load_any(static_cast<const unsigned char *>(r.b) + (long long)(i - nl) * r.stride);
    }
}

__global__ void scatter_calls_kernel(const CallRow *calls, const __grid_constant__ CallRowsParam P, int n_calls, int N,
                                     bool inverse, const float *src, long long spitch)
{
    const int k = blockIdx.y;
    if (k >= n_calls) return;
    const CallRow r = calls ? calls[k] : P.r[k];
    const float *row = src + (long long)k * spitch;
    const int nl = (N + 1) / 2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        if (inverse || i < nl)
            store_any(static_cast<unsigned char *>(r.c) + (long long)i * r.stride, row[i]);
        else
            store_any(static_cast<unsigned char *>(r.h) + (long long)(i - nl) * r.stride, row[i]);
    }
}

// Combined strided 1D calls in one launch, one block per call: the call's
// samples (forward: N at a; inverse: L at a, H at b) are gathered into
// shared memory, lifted there as per-thread windows of one line
// (dwt_recur.cuh), and stored back at the call's destinations (forward: L
// at c, H at h; inverse: N samples at c), all `stride` bytes apart.
constexpr int kCalls1dThreads = 512;
constexpr int kCalls1dUnroll = 8;  // loads (stores) in flight per thread

template <int NS, bool INV>
__global__ void __launch_bounds__(kCalls1dThreads) calls_1d_kernel(const CallRow *calls,
                                                                   const __grid_constant__ CallRowsParam P,
                                                                   int n_calls, int N, const Wavelet W)
{
    extern __shared__ float sm1[];
    const int k = blockIdx.x;
    if (k >= n_calls) return;
    const CallRow r = calls ? calls[k] : P.r[k];
    float *A = sm1, *B = sm1 + N;
    const int nl = (N + 1) / 2, tid = threadIdx.x, nt = blockDim.x;
    const unsigned char *a = static_cast<const unsigned char *>(r.a), *b = static_cast<const unsigned char *>(r.b);
    unsigned char *c = static_cast<unsigned char *>(r.c), *h = static_cast<unsigned char *>(r.h);
    const long long st = r.stride;
    // sample i of the source / destination (forward: N at a / L at c, H at
    // h; inverse: L at a, H at b / N at c)
    auto src = [&](int i) { return (!INV || i < nl) ? a + (long long)i * st : b + (long long)(i - nl) * st; };
    auto dst = [&](int i) { return (INV || i < nl) ? c + (long long)i * st : h + (long long)(i - nl) * st; };
    const bool aligned = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) |
                           reinterpret_cast<uintptr_t>(c) | reinterpret_cast<uintptr_t>(h) | uintptr_t(st)) & 3) == 0;
    pdl_wait();
    for (int i0 = tid; i0 < N; i0 += kCalls1dUnroll * nt) {
        float v[kCalls1dUnroll];
#pragma unroll
        for (int u = 0; u < kCalls1dUnroll; ++u) {
            const int i = i0 + u * nt;
            if (i < N) v[u] = aligned ? __ldg(reinterpret_cast<const float *>(src(i))) : load_any(src(i));
        }
#pragma unroll
        for (int u = 0; u < kCalls1dUnroll; ++u)
            if (i0 + u * nt < N) A[i0 + u * nt] = v[u];
    }
    __syncthreads();
    recur::pass<NS, INV>(A, 0, 1, B, 0, 1, 1, N, W, tid, nt);
    __syncthreads();
    for (int i = tid; i < N; i += nt) {
        if (aligned)
            *reinterpret_cast<float *>(dst(i)) = B[i];
        else
            store_any(dst(i), B[i]);
    }
}

// Interleaved channels (pixel = `channels` floats) <-> one compact plane per
// channel, plane c at planes + c * plane_stride (pitch in floats).
__global__ void deinterleave_kernel(const unsigned char *src, long long src_pitch, int channels, int w, int h,
                                    float *planes, long long pitch, long long plane_stride)
{
    const long long n = (long long)w * h * channels;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const long long row = k / ((long long)w * channels);
        const int e = int(k - row * w * channels);  // float index within the row: x * channels + c
        const int x = e / channels, c = e - x * channels;
        planes[c * plane_stride + row * pitch + x] = load_any(src + row * src_pitch + (long long)e * 4);
    }
}

__global__ void interleave_kernel(const float *planes, long long pitch, long long plane_stride, int channels, int w,
                                  int h, unsigned char *dst, long long dst_pitch)
{
    const long long n = (long long)w * h * channels;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const long long row = k / ((long long)w * channels);
        const int e = int(k - row * w * channels);
        const int x = e / channels, c = e - x * channels;
        store_any(dst + row * dst_pitch + (long long)e * 4, planes[c * plane_stride + row * pitch + x]);
    }
}

int grid_for(long long n, int block)
{
    long long g = (n + block - 1) / block;
    if (g > 152LL * 32) g = 152LL * 32;
    if (g < 1) g = 1;
    return int(g);
}

// Device-to-device copy of `rows` rows of `width` bytes by one warp per
// block through a small ring of shared-memory buffers with TMA bulk copies
// (kBulkBufs - 1 loads in flight), so that a block fits beside level kernels
// that fill an SM's registers and most of its shared memory: a copy on
// another stream then streams during the latency-bound smaller levels
// instead of waiting for free SM slots.  Every 16-byte aligned; waits are
// bounded (the error word on a timeout, after which the block only drains
// its stores).
constexpr int kBulkBufs = 4;
constexpr int kBulkPiece = 4096;  // bytes per buffer
constexpr int kBulkSmem = kBulkBufs * kBulkPiece + kBulkBufs * 8;

__global__ void __launch_bounds__(32) bulk_copy_rows_kernel(const unsigned char *src, long long spitch,
                                                            unsigned char *dst, long long dpitch, long long width,
                                                            long long rows, int *err)
{
    extern __shared__ __align__(128) unsigned char sm[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + kBulkBufs * kBulkPiece);
    const int lane = threadIdx.x;
    if (lane == 0) {
        for (int b = 0; b < kBulkBufs; ++b) mbar_init(&bar[b], 1);
        fence_mbar_init();
    }
    __syncwarp();
    const long long per_row = (width + kBulkPiece - 1) / kBulkPiece;
    const long long total = per_row * rows;
    // this block's pieces: blockIdx.x, + gridDim.x, ...; i-th of them
    auto piece = [&](long long i, const unsigned char *&s, unsigned char *&d, uint32_t &bytes) {
        const long long c = blockIdx.x + i * gridDim.x;
        const long long r = c / per_row, off = (c % per_row) * kBulkPiece;
        s = src + r * spitch + off;
        d = dst + r * dpitch + off;
        bytes = uint32_t(width - off < kBulkPiece ? width - off : kBulkPiece);
    };
    const long long mine = total > blockIdx.x ? (total - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
    auto load = [&](long long i) {
        const unsigned char *s;
        unsigned char *d;
        uint32_t bytes;
        piece(i, s, d, bytes);
        const int b = int(i % kBulkBufs);
        mbar_arrive_expect_tx(&bar[b], bytes);
        bulk_g2s(sm + b * kBulkPiece, s, bytes, &bar[b]);
    };
    long long issued = mine < kBulkBufs - 1 ? mine : kBulkBufs - 1;
    if (lane == 0)
        for (long long i = 0; i < issued; ++i) load(i);
    __syncwarp();
    for (long long i = 0; i < mine; ++i) {
        const int b = int(i % kBulkBufs);
        if (!__all_sync(0xffffffffu, mbar_wait_bounded(&bar[b], uint32_t(i / kBulkBufs) & 1u))) {
            // give up: raise the error and wait (bounded) for the loads still
            // in flight before the block's shared memory goes away
            if (lane == 0) {
                if (err) atomicCAS(err, 0, int(kErrWaitTimeout));
                for (long long j = i; j < issued; ++j)
                    mbar_wait_bounded(&bar[j % kBulkBufs], uint32_t(j / kBulkBufs) & 1u);
            }
            break;
        }
        if (lane == 0) {
            const unsigned char *s;
            unsigned char *d;
            uint32_t bytes;
            piece(i, s, d, bytes);
            fence_proxy_async_smem();
            bulk_s2g(d, sm + b * kBulkPiece, bytes);
            bulk_commit();
            if (issued < mine) {
                // the buffer of piece `issued` was read by the store of piece
                // i - 1: at most the store just issued may still read
                bulk_wait_read<1>();
                load(issued++);
            }
        }
        issued = __shfl_sync(0xffffffffu, issued, 0);
    }
    if (lane == 0) bulk_wait_all();
    __syncwarp();
}

}  // namespace

cudaError_t launch_repack(const void *src, long long sx, long long sy, int ox, int oy, float *dst,
                          long long dpitch, cudaStream_t s)
{
    if ((long long)ox * oy == 0) return cudaSuccess;
    repack_kernel<<<grid_for((long long)ox * oy, 256), 256, 0, s>>>(
        static_cast<const unsigned char *>(src), sx, sy, ox, oy, dst, dpitch);
    return cudaGetLastError();
}

cudaError_t launch_unpack(const float *src, long long spitch, void *dst, long long sx, long long sy,
                          int ox, int oy, cudaStream_t s)
{
    if ((long long)ox * oy == 0) return cudaSuccess;
    unpack_kernel<<<grid_for((long long)ox * oy, 256), 256, 0, s>>>(
        src, spitch, static_cast<unsigned char *>(dst), sx, sy, ox, oy);
    return cudaGetLastError();
}

cudaError_t launch_copy_rows(void *dst, long long dpitch, const void *src, long long spitch, long long width,
                             long long rows, cudaStream_t s)
{
    return launch_copy_rows_ctas(dst, dpitch, src, spitch, width, rows, s, 0);
}

cudaError_t launch_copy_rows_dev(void *dst, long long dpitch, const void *src, long long spitch, long long width,
                                 long long rows, cudaStream_t s)
{
    // device to device: enough blocks to stream at HBM speed (8 per SM)
    static const int ctas = [] {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 152;
        return 8 * sms;
    }();
    return launch_copy_rows_ctas(dst, dpitch, src, spitch, width, rows, s, ctas);
}

cudaError_t launch_copy_rows_bulk(void *dst, long long dpitch, const void *src, long long spitch, long long width,
                                  long long rows, cudaStream_t s, int *err)
{
    if (width <= 0 || rows <= 0) return cudaSuccess;
    const uintptr_t a = reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) |
                        uintptr_t(dpitch) | uintptr_t(spitch) | uintptr_t(width);
    if ((a & 15) != 0) return launch_copy_rows_dev(dst, dpitch, src, spitch, width, rows, s);
    // 4 blocks per SM: one fits beside a full level kernel, the others run
    // as the level kernels drain
    static const int ctas = [] {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 152;
        const char *e = getenv("DWT_GPU_BULK_COPY_CTAS");
        const int v = e ? atoi(e) : 0;
        return (v > 0 && v <= 32 ? v : 4) * sms;
    }();
    const long long pieces = (width + kBulkPiece - 1) / kBulkPiece * rows;
    const int grid = int(std::min<long long>(pieces, ctas));
    bulk_copy_rows_kernel<<<grid, 32, kBulkSmem, s>>>(static_cast<const unsigned char *>(src), spitch,
                                                     static_cast<unsigned char *>(dst), dpitch, width, rows, err);
    return cudaGetLastError();
}

cudaError_t launch_copy_rows_ctas(void *dst, long long dpitch, const void *src, long long spitch, long long width,
                                  long long rows, cudaStream_t s, int ctas_override)
{
    if (width <= 0 || rows <= 0) return cudaSuccess;
    if (rows > INT32_MAX) return cudaErrorInvalidValue;
    const uintptr_t a = reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) |
                        uintptr_t(dpitch) | uintptr_t(spitch) | uintptr_t(width);
    const int vb = (a & 15) == 0 ? 16 : (a & 3) == 0 ? 4 : 1;
    const long long per_row = width / vb;
    if (per_row > INT32_MAX) return cudaErrorInvalidValue;
    // 64 blocks of 256 threads in all (measured best for pageable host frames
    // of 16384^2 against 32, 128 and 304; DWT_GPU_COPY_CTAS overrides), each
    // moving 4 x 256 elements of a row per step: enough bytes in flight for
    // the host link, few blocks to wait for free SM slots among the band
    // kernels
    static const int host_ctas = [] {
        const char *e = getenv("DWT_GPU_COPY_CTAS");
        const int v = e ? atoi(e) : 0;
        return v > 0 ? v : 64;
    }();
    const int ctas = ctas_override > 0 ? ctas_override : host_ctas;
    const int gx = int(std::min<long long>((per_row + 1023) / 1024, 16));
    const int gy = int(std::min<long long>(rows, std::max(1, ctas / gx)));
    const dim3 grid(gx, gy);
    const auto *sp = static_cast<const unsigned char *>(src);
    auto *dp = static_cast<unsigned char *>(dst);
    if (vb == 16)
        copy_rows_kernel<uint4><<<grid, 256, 0, s>>>(sp, spitch, dp, dpitch, int(per_row), int(rows));
    else if (vb == 4)
        copy_rows_kernel<uint32_t><<<grid, 256, 0, s>>>(sp, spitch, dp, dpitch, int(per_row), int(rows));
    else
        copy_rows_kernel<unsigned char><<<grid, 256, 0, s>>>(sp, spitch, dp, dpitch, int(per_row), int(rows));
    return cudaGetLastError();
}

cudaError_t launch_deinterleave(const void *src, long long src_pitch_bytes, int channels, int w, int h,
                                float *planes, long long pitch, long long plane_stride, cudaStream_t s)
{
    const long long n = (long long)w * h * channels;
    if (n == 0) return cudaSuccess;
    deinterleave_kernel<<<grid_for(n, 256), 256, 0, s>>>(static_cast<const unsigned char *>(src), src_pitch_bytes,
                                                          channels, w, h, planes, pitch, plane_stride);
    return cudaGetLastError();
}

cudaError_t launch_interleave(const float *planes, long long pitch, long long plane_stride, int channels, int w,
                              int h, void *dst, long long dst_pitch_bytes, cudaStream_t s)
{
    const long long n = (long long)w * h * channels;
    if (n == 0) return cudaSuccess;
    interleave_kernel<<<grid_for(n, 256), 256, 0, s>>>(planes, pitch, plane_stride, channels, w, h,
                                                        static_cast<unsigned char *>(dst), dst_pitch_bytes);
    return cudaGetLastError();
}

cudaError_t launch_gather_signals(const void *base, int N, long long stride, long long count, int group,
                                  long long group_stride, long long lane_stride, float *dst,
                                  long long dpitch, cudaStream_t s)
{
    if ((long long)N * count == 0) return cudaSuccess;
    gather_signals_kernel<<<grid_for((long long)N * count, 256), 256, 0, s>>>(
        static_cast<const unsigned char *>(base), N, stride, count, group, group_stride, lane_stride, dst,
        dpitch);
    return cudaGetLastError();
}

cudaError_t launch_scatter_signals(const float *src, long long spitch, int N, void *base, long long stride,
                                   long long count, int group, long long group_stride,
                                   long long lane_stride, cudaStream_t s)
{
    if ((long long)N * count == 0) return cudaSuccess;
    scatter_signals_kernel<<<grid_for((long long)N * count, 256), 256, 0, s>>>(
        src, spitch, N, static_cast<unsigned char *>(base), stride, count, group, group_stride,
        lane_stride);
    return cudaGetLastError();
}

// The rows as a kernel parameter when they fit (and no device array is given).
static bool call_rows_param(const CallRow *calls, const CallRow *host_calls, int n_calls, CallRowsParam &P)
{
    if (calls) return true;
    if (!host_calls || n_calls > kCallRowsParam) return false;
    for (int k = 0; k < n_calls; ++k) P.r[k] = host_calls[k];
    return true;
}

cudaError_t launch_gather_calls(const CallRow *calls, const CallRow *host_calls, int n_calls, int N, bool inverse,
                                float *dst, long long dpitch, int h_off, cudaStream_t s)
{
    if (n_calls <= 0 || N <= 0) return cudaSuccess;
    if (n_calls > 65535) return cudaErrorInvalidValue;
    CallRowsParam P;
    if (!call_rows_param(calls, host_calls, n_calls, P)) return cudaErrorInvalidValue;
    const dim3 grid(unsigned(std::min(ceil_div(N, 256), 64)), unsigned(n_calls));
    gather_calls_kernel<<<grid, 256, 0, s>>>(calls, P, n_calls, N, inverse, dst, dpitch, h_off);
    return cudaGetLastError();
}

cudaError_t launch_scatter_calls(const CallRow *calls, const CallRow *host_calls, int n_calls, int N, bool inverse,
                                 const float *src, long long spitch, cudaStream_t s)
{
    if (n_calls <= 0 || N <= 0) return cudaSuccess;
    if (n_calls > 65535) return cudaErrorInvalidValue;
    CallRowsParam P;
    if (!call_rows_param(calls, host_calls, n_calls, P)) return cudaErrorInvalidValue;
    const dim3 grid(unsigned(std::min(ceil_div(N, 256), 64)), unsigned(n_calls));
    scatter_calls_kernel<<<grid, 256, 0, s>>>(calls, P, n_calls, N, inverse, src, spitch);
    return cudaGetLastError();
}

cudaError_t launch_calls_1d(const CallRow *calls, const CallRow *host_calls, int n_calls, int N, int wavelet,
                            bool inverse, cudaStream_t s)
{
    if (n_calls <= 0 || N <= 0) return cudaSuccess;
    if (N > kCalls1dMaxN || n_calls > 65535 * 32) return cudaErrorInvalidValue;
    CallRowsParam P;
    if (!call_rows_param(calls, host_calls, n_calls, P)) return cudaErrorInvalidValue;
    static const cudaError_t configured = [] {
        cudaError_t e = cudaSuccess;
        for (auto k : {calls_1d_kernel<4, false>, calls_1d_kernel<4, true>, calls_1d_kernel<2, false>,
                       calls_1d_kernel<2, true>})
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 8 * kCalls1dMaxN);
        return e;
    }();
    if (configured != cudaSuccess) return configured;
    const Wavelet W = make_wavelet(wavelet, inverse);
    const size_t smem = size_t(8) * N;
    const dim3 g(static_cast<unsigned>(n_calls)), b(kCalls1dThreads);
    if (wavelet == CDF97)
        return inverse ? launch_pdl(calls_1d_kernel<4, true>, g, b, smem, s, calls, P, n_calls, N, W)
                       : launch_pdl(calls_1d_kernel<4, false>, g, b, smem, s, calls, P, n_calls, N, W);
    return inverse ? launch_pdl(calls_1d_kernel<2, true>, g, b, smem, s, calls, P, n_calls, N, W)
                   : launch_pdl(calls_1d_kernel<2, false>, g, b, smem, s, calls, P, n_calls, N, W);
}

size_t sparse_tail_smem(int ox, int oy, int j0)
{
    const int fx = ceil_div_pow2(ox, j0), fy = ceil_div_pow2(oy, j0);
    return size_t(fx | 1) * fy * 4 * 2;
}

cudaError_t launch_sparse_tail(bool inverse, float *f, long long pitch, int ox, int oy, int ix, int iy, int j0,
                               int j1, int wavelet, cudaStream_t s)
{
    const size_t smem = sparse_tail_smem(ox, oy, j0);
    if (smem > kSparseTailSmem || j1 <= j0) return cudaErrorInvalidValue;
    static const cudaError_t configured = [] {
        cudaError_t e = cudaSuccess;
        for (auto k : {sparse_tail_kernel<4, false>, sparse_tail_kernel<4, true>, sparse_tail_kernel<2, false>,
                       sparse_tail_kernel<2, true>})
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kSparseTailSmem);
        return e;
    }();
    if (configured != cudaSuccess) return configured;
    const Wavelet W = make_wavelet(wavelet, inverse);
    const dim3 g(1), b(kTailThreads);
    if (wavelet == CDF97) {
        if (inverse)
            sparse_tail_kernel<4, true><<<g, b, smem, s>>>(f, pitch, ox, oy, ix, iy, j0, j1, W);
        else
            sparse_tail_kernel<4, false><<<g, b, smem, s>>>(f, pitch, ox, oy, ix, iy, j0, j1, W);
    } else {
        if (inverse)
            sparse_tail_kernel<2, true><<<g, b, smem, s>>>(f, pitch, ox, oy, ix, iy, j0, j1, W);
        else
            sparse_tail_kernel<2, false><<<g, b, smem, s>>>(f, pitch, ox, oy, ix, iy, j0, j1, W);
    }
    return cudaGetLastError();
}

cudaError_t launch_zero_rects(float *f, long long pitch, const ZeroRects &R, cudaStream_t s)
{
    if (R.n <= 0 || R.total_rows <= 0) return cudaSuccess;
    const int grid = std::min(R.total_rows, 152 * 16);
    zero_rects_kernel<<<grid, 256, 0, s>>>(f, pitch, R);
    return cudaGetLastError();
}

// Sparse-frame level on a compact frame `f` (pitch in floats), in place, the
// reference driver's exact sequence.  tmp holds max(lines) * max(len) floats.
cudaError_t sparse_forward_level(float *f, long long pitch, int osx, int osy, int odx, int ody, int isx,
                                 int isy, int zero_padding, int wavelet, float *tmp, cudaStream_t s)
{
    const Wavelet W = make_wavelet(wavelet, false);
    lines_forward_kernel<<<ceil_div(osy, 128), 128, 0, s>>>(f, pitch, 1, osy, isx, odx, tmp, W);
    lines_forward_kernel<<<ceil_div(osx, 128), 128, 0, s>>>(f, 1, pitch, osx, isy, ody, tmp, W);
    if (zero_padding) {
        zero_forward_kernel<<<ceil_div(osy, 128), 128, 0, s>>>(f, pitch, 1, osy, isx, odx, osx - odx, odx);
        zero_forward_kernel<<<ceil_div(osx, 128), 128, 0, s>>>(f, 1, pitch, osx, isy, ody, osy - ody, ody);
    }
    return cudaGetLastError();
}

cudaError_t sparse_inverse_level(float *f, long long pitch, int osx, int osy, int odx, int ody, int idx,
                                 int idy, int zero_padding, int wavelet, float *tmp, cudaStream_t s)
{
    const Wavelet W = make_wavelet(wavelet, true);
    lines_inverse_kernel<<<ceil_div(ody, 128), 128, 0, s>>>(f, pitch, 1, ody, idx, osx, tmp, W);
    lines_inverse_kernel<<<ceil_div(odx, 128), 128, 0, s>>>(f, 1, pitch, odx, idy, osy, tmp, W);
    if (zero_padding) {
        zero_inverse_kernel<<<ceil_div(ody, 128), 128, 0, s>>>(f, pitch, 1, ody, idx, odx);
        zero_inverse_kernel<<<ceil_div(odx, 128), 128, 0, s>>>(f, 1, pitch, odx, idy, ody);
    }
    return cudaGetLastError();
}

}  // namespace dwt
