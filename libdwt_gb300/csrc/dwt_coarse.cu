// All remaining coarse levels of one image in a single CTA.
//
// Once the LL band is small, each further level has too little work to fill
// the GPU and a launch per level costs more than the level itself.  This
// kernel loads the band into shared memory and runs every remaining level
// there.  A pass gives each line (row or column) to one warp, which holds up
// to 256 samples in registers (8 per lane, mirrored past the end of the
// line) and runs the lifting steps with warp shuffles, the same per-sample
// arithmetic as the reference (x + c*(l + r), symmetric extension, scaling).
// Each pass writes its result transposed and deinterleaved into the other
// buffer, so the column pass reads its lines as rows too.  The forward writes
// each level's detail bands and the final LL to the output frame; the
// inverse reads them and writes the reconstructed band.
#include "dwt_coarse.cuh"

#include <algorithm>

namespace dwt {

namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr int kV = 8;  // samples per lane: one warp holds 256 samples of a line
constexpr unsigned kAll = 0xffffffffu;

// Forward lifting of one line of length n (2 <= n <= 252) held by a warp,
// sample 8*lane + k in x[k]; samples past the end hold their mirror images.
// Every lifting step is applied uniformly; the left neighbour of sample 0 is
// sample 1 (symmetric extension), and the missing right neighbour of the
// warp's last sample only disturbs samples >= 252 - 4 steps, beyond n + 3.
template <int NS>
__device__ __forceinline__ void line_forward(float x[kV], const Wavelet &W, int lane)
{
#pragma unroll
    for (int s = 0; s < NS; s += 2) {
        const float nx = __shfl_down_sync(kAll, x[0], 1);
#pragma unroll
        for (int k = 1; k < kV - 1; k += 2) x[k] = lift(x[k], W.c[s], x[k - 1], x[k + 1]);
        x[kV - 1] = lift(x[kV - 1], W.c[s], x[kV - 2], nx);
        float pv = __shfl_up_sync(kAll, x[kV - 1], 1);
        if (lane == 0) pv = x[1];
        x[0] = lift(x[0], W.c[s + 1], pv, x[1]);
#pragma unroll
        for (int k = 2; k < kV; k += 2) x[k] = lift(x[k], W.c[s + 1], x[k - 1], x[k + 1]);
    }
#pragma unroll
    for (int k = 0; k < kV; ++k) x[k] = fmul(x[k], (k & 1) ? W.zeta_o : W.zeta_e);
}

template <int NS>
__device__ __forceinline__ void line_inverse(float x[kV], const Wavelet &W, int lane)
{
#pragma unroll
    for (int k = 0; k < kV; ++k) x[k] = fmul(x[k], (k & 1) ? W.zeta_e : W.zeta_o);
#pragma unroll
    for (int s = 0; s < NS; s += 2) {
        float pv = __shfl_up_sync(kAll, x[kV - 1], 1);
        if (lane == 0) pv = x[1];
        x[0] = lift(x[0], W.c[s], pv, x[1]);
#pragma unroll
        for (int k = 2; k < kV; k += 2) x[k] = lift(x[k], W.c[s], x[k - 1], x[k + 1]);
        const float nx = __shfl_down_sync(kAll, x[0], 1);
#pragma unroll
        for (int k = 1; k < kV - 1; k += 2) x[k] = lift(x[k], W.c[s + 1], x[k - 1], x[k + 1]);
        x[kV - 1] = lift(x[kV - 1], W.c[s + 1], x[kV - 2], nx);
    }
}

// One forward pass over `nl` lines of length n: line l sample i read from
// src[l*ls + i]; results deinterleaved and transposed into dst: sample i of
// line l goes to dst[(i even ? i/2 : nd + i/2) * dp + l], nd = ceil(n/2).
// The lane's mirrored load offsets and store rows depend only on n, so they
// are computed once per pass.
template <int NS>
__device__ __forceinline__ void pass_forward(const float *src, int ls, float *dst, int dp, int nl, int n,
                                             const Wavelet &W, int warp, int lane)
{
    const int nd = (n + 1) >> 1;
    if (n == 1) {
        for (int l = threadIdx.x; l < nl; l += blockDim.x) dst[l] = fmul(src[l * ls], W.n1_fwd);
        return;
    }
    int ld[kV], st[kV];
#pragma unroll
    for (int k = 0; k < kV; ++k) {
        const int i = kV * lane + k;
        ld[k] = mirror(i, n);
        st[k] = i < n ? ((k & 1) ? nd + (i >> 1) : (i >> 1)) * dp : -1;
    }
    for (int l = warp; l < nl; l += kWarps) {
        const float *line = src + l * ls;
        float x[kV];
#pragma unroll
        for (int k = 0; k < kV; ++k) x[k] = line[ld[k]];
        line_forward<NS>(x, W, lane);
#pragma unroll
        for (int k = 0; k < kV; ++k)
            if (st[k] >= 0) dst[st[k] + l] = x[k];
    }
}

// One inverse pass: line l holds L samples at src[l*ls + j] (j < nd) and H
// samples at src[l*ls + nd + j]; rebuilt samples transposed into dst[i*dp + l].
template <int NS>
__device__ __forceinline__ void pass_inverse(const float *src, int ls, float *dst, int dp, int nl, int n,
                                             const Wavelet &W, int warp, int lane)
{
    const int nd = (n + 1) >> 1;
    if (n == 1) {
        for (int l = threadIdx.x; l < nl; l += blockDim.x) dst[l] = fmul(src[l * ls], W.n1_inv);
        return;
    }
    int ld[kV], st[kV];
#pragma unroll
    for (int k = 0; k < kV; ++k) {
        const int i = kV * lane + k;
        const int m = mirror(i, n);
        ld[k] = (m & 1) ? nd + (m >> 1) : (m >> 1);
        st[k] = i < n ? i * dp : -1;
    }
    for (int l = warp; l < nl; l += kWarps) {
        const float *line = src + l * ls;
        float x[kV];
#pragma unroll
        for (int k = 0; k < kV; ++k) x[k] = line[ld[k]];
        line_inverse<NS>(x, W, lane);
#pragma unroll
        for (int k = 0; k < kV; ++k)
            if (st[k] >= 0) dst[st[k] + l] = x[k];
    }
}

// A: the band, row-major with pitch P; B: its transpose, pitch PT.
template <int NS>
__global__ void __launch_bounds__(kThreads)
coarse_forward_kernel(const float *in, long long in_pitch, int w0, int h0, int levels, float *out,
                      long long out_pitch, const Wavelet W)
{
    extern __shared__ float sm[];
    const int P = w0 + 1, PT = h0 + 1;
    float *A = sm, *B = sm + P * h0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int y = threadIdx.x >> 5; y < h0; y += kWarps)
        for (int x = threadIdx.x & 31; x < w0; x += 32) A[y * P + x] = in[y * in_pitch + x];
    __syncthreads();
    int w = w0, h = h0;
    for (int lvl = 0; lvl < levels; ++lvl) {
        const int wd = (w + 1) >> 1, hd = (h + 1) >> 1;
        pass_forward<NS>(A, P, B, PT, h, w, W, warp, lane);  // rows -> columns of B
        __syncthreads();
        pass_forward<NS>(B, PT, A, P, w, h, W, warp, lane);  // columns -> rows of A
        __syncthreads();
        for (int y = warp; y < h; y += kWarps)
            for (int x = (y < hd ? wd : 0) + lane; x < w; x += 32) out[y * out_pitch + x] = A[y * P + x];
        w = wd;
        h = hd;
    }
    for (int y = warp; y < h; y += kWarps)
        for (int x = lane; x < w; x += 32) out[y * out_pitch + x] = A[y * P + x];
}

template <int NS>
__global__ void __launch_bounds__(kThreads)
coarse_inverse_kernel(const float *in, long long in_pitch, int w0, int h0, int levels, float *out,
                      long long out_pitch, const Wavelet W)
{
    extern __shared__ float sm[];
    const int P = w0 + 1, PT = h0 + 1;
    float *A = sm, *B = sm + P * h0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int y = threadIdx.x >> 5; y < h0; y += kWarps)
        for (int x = threadIdx.x & 31; x < w0; x += 32) A[y * P + x] = in[y * in_pitch + x];
    __syncthreads();
    for (int lvl = levels - 1; lvl >= 0; --lvl) {
        int w = w0, h = h0;
        for (int k = 0; k < lvl; ++k) {
            w = (w + 1) >> 1;
            h = (h + 1) >> 1;
        }
        // rows first (src/libdwt.c:6706-6717): rows of A -> columns of B
        pass_inverse<NS>(A, P, B, PT, h, w, W, warp, lane);
        __syncthreads();
        // then columns: columns of B hold the L rows then the H rows
        pass_inverse<NS>(B, PT, A, P, w, h, W, warp, lane);
        __syncthreads();
    }
    for (int y = warp; y < h0; y += kWarps)
        for (int x = lane; x < w0; x += 32) out[y * out_pitch + x] = A[y * P + x];
}

template <typename K>
cudaError_t configure(K kernel)
{
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kCoarseSmem);
}

}  // namespace

cudaError_t launch_coarse(bool inverse, const float *in, long long in_pitch, int w, int h, int levels,
                          float *out, long long out_pitch, int wavelet, cudaStream_t s)
{
    static bool configured = false;
    if (!configured) {
        cudaError_t e = configure(coarse_forward_kernel<4>);
        if (e == cudaSuccess) e = configure(coarse_inverse_kernel<4>);
        if (e == cudaSuccess) e = configure(coarse_forward_kernel<2>);
        if (e == cudaSuccess) e = configure(coarse_inverse_kernel<2>);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    if (!coarse_fits(w, h)) return cudaErrorInvalidValue;
    const Wavelet W = make_wavelet(wavelet, inverse);
    const size_t smem = size_t(4) * ((w + 1) * h + (h + 1) * w);
    if (wavelet == CDF97) {
        if (inverse)
            coarse_inverse_kernel<4><<<1, kThreads, smem, s>>>(in, in_pitch, w, h, levels, out, out_pitch, W);
        else
            coarse_forward_kernel<4><<<1, kThreads, smem, s>>>(in, in_pitch, w, h, levels, out, out_pitch, W);
    } else {
        if (inverse)
            coarse_inverse_kernel<2><<<1, kThreads, smem, s>>>(in, in_pitch, w, h, levels, out, out_pitch, W);
        else
            coarse_forward_kernel<2><<<1, kThreads, smem, s>>>(in, in_pitch, w, h, levels, out, out_pitch, W);
    }
    return cudaGetLastError();
}

}  // namespace dwt
