// Layout repacking and the per-line sparse-frame path (see dwt_generic.cu).
#pragma once

#include "dwt_common.cuh"

namespace dwt {

// caller layout (byte strides, any alignment) -> compact float frame
cudaError_t launch_repack(const void *src, long long sx, long long sy, int ox, int oy, float *dst,
                          long long dpitch, cudaStream_t s);
// compact float frame -> caller layout; touches only the frame's samples
cudaError_t launch_unpack(const float *src, long long spitch, void *dst, long long sx, long long sy,
                          int ox, int oy, cudaStream_t s);

// `rows` rows of `width` bytes, pitches in bytes, by a kernel: for host
// memory the GPU addresses directly (pageable memory under address
// translation services), where it keeps the copy asynchronous to the host.
cudaError_t launch_copy_rows(void *dst, long long dpitch, const void *src, long long spitch, long long width,
                             long long rows, cudaStream_t s);
// The same between device frames, with enough blocks for HBM bandwidth (the
// copy engines move 2D device-to-device copies far slower).
cudaError_t launch_copy_rows_dev(void *dst, long long dpitch, const void *src, long long spitch, long long width,
                                 long long rows, cudaStream_t s);
// The same through TMA bulk copies by one-warp blocks with 16 KB of shared
// memory, which fit beside full level kernels (a copy on a second stream);
// 16-byte aligned frames only, else launch_copy_rows_dev.  err: device error
// word of a bounded wait that gave up (may be null).
cudaError_t launch_copy_rows_bulk(void *dst, long long dpitch, const void *src, long long spitch, long long width,
                                  long long rows, cudaStream_t s, int *err);
cudaError_t launch_copy_rows_ctas(void *dst, long long dpitch, const void *src, long long spitch, long long width,
                                  long long rows, cudaStream_t s, int ctas);

// strided signal bank <-> compact rows (one signal per row)
// Interleaved channels (pixel = `channels` floats, rows src_pitch_bytes
// apart) <-> one compact plane per channel (plane c at planes + c *
// plane_stride, row pitch `pitch` floats).
cudaError_t launch_deinterleave(const void *src, long long src_pitch_bytes, int channels, int w, int h,
                                float *planes, long long pitch, long long plane_stride, cudaStream_t s);
cudaError_t launch_interleave(const float *planes, long long pitch, long long plane_stride, int channels, int w,
                              int h, void *dst, long long dst_pitch_bytes, cudaStream_t s);

cudaError_t launch_gather_signals(const void *base, int N, long long stride, long long count, int group,
                                  long long group_stride, long long lane_stride, float *dst,
                                  long long dpitch, cudaStream_t s);
cudaError_t launch_scatter_signals(const float *src, long long spitch, int N, void *base, long long stride,
                                   long long count, int group, long long group_stride,
                                   long long lane_stride, cudaStream_t s);

// One strided 1D call of a combined batch: its sources (a; the inverse's H
// from b), its destinations (c; the forward's H to h) and its byte stride.
struct CallRow {
    const void *a, *b;
    void *c, *h;
    long long stride;
};
// Up to kCallRowsParam calls travel as a kernel parameter (no descriptor
// upload); larger batches read a device array.
constexpr int kCallRowsParam = 64;
struct CallRowsParam {
    CallRow r[kCallRowsParam];
};
// The calls' signals (N samples each) into the rows of a compact frame
// (inverse: L at the row's start, H from h_off), and the rows' results back.
// `calls`: a device array of the n_calls rows, or null when n_calls <=
// kCallRowsParam and `host_calls` holds them.
cudaError_t launch_gather_calls(const CallRow *calls, const CallRow *host_calls, int n_calls, int N, bool inverse,
                                float *dst, long long dpitch, int h_off, cudaStream_t s);
cudaError_t launch_scatter_calls(const CallRow *calls, const CallRow *host_calls, int n_calls, int N, bool inverse,
                                 const float *src, long long spitch, cudaStream_t s);
// The calls transformed in one launch, one block per call, in shared memory
// (N <= kCalls1dMaxN); `calls` / `host_calls` as above.
constexpr int kCalls1dMaxN = 24576;
cudaError_t launch_calls_1d(const CallRow *calls, const CallRow *host_calls, int n_calls, int N, int wavelet,
                            bool inverse, cudaStream_t s);

// The per-line levels of a sparse frame with zero padding in one CTA, the
// frame of level j0 held in shared memory: forward levels j0 .. j1-1 or
// inverse levels j1 .. j0+1.  Only when sparse_tail_smem(ox, oy, j0) fits
// kSparseTailSmem (cudaErrorInvalidValue otherwise).
constexpr size_t kSparseTailSmem = 200 * 1024;
size_t sparse_tail_smem(int ox, int oy, int j0);
cudaError_t launch_sparse_tail(bool inverse, float *f, long long pitch, int ox, int oy, int ix, int iy, int j0,
                               int j1, int wavelet, cudaStream_t s);

// Rectangles of a frame to fill with zeros (at most kMaxZeroRects; the rows
// of rectangle k are rows first_row[k] .. of the flattened list).
constexpr int kMaxZeroRects = 128;
struct ZeroRects {
    int n, total_rows;
    int x0[kMaxZeroRects], y0[kMaxZeroRects], w[kMaxZeroRects], first_row[kMaxZeroRects];
};
cudaError_t launch_zero_rects(float *f, long long pitch, const ZeroRects &R, cudaStream_t s);

// One level of a sparse frame (outer > inner), in place on a compact frame.
cudaError_t sparse_forward_level(float *f, long long pitch, int osx, int osy, int odx, int ody, int isx,
                                 int isy, int zero_padding, int wavelet, float *tmp, cudaStream_t s);
cudaError_t sparse_inverse_level(float *f, long long pitch, int osx, int osy, int odx, int ody, int idx,
                                 int idy, int zero_padding, int wavelet, float *tmp, cudaStream_t s);

}  // namespace dwt
