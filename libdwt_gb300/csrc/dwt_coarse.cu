// All remaining coarse levels of one image in a single CTA.
//
// Once the LL band is small, each further level has too little work to fill
// the GPU and a launch per level costs more than the level itself.  This
// kernel loads the band into shared memory and runs every remaining level
// there, each level as a row pass and a column pass of per-thread lifting
// recurrences (one thread per line segment, dwt_recur.cuh) between two
// row-major buffers with an odd pitch, so neither pass has bank conflicts
// and nothing is transposed.  The forward writes each level's detail bands
// and the final LL to the output frame; the inverse reads them and writes
// the reconstructed band.
#include "dwt_coarse.cuh"

#include <algorithm>

namespace dwt {

namespace {

// 512 threads and windows of 2 output pairs: the levels here are
// latency-bound, so short per-thread dependency chains and a smaller
// barrier beat fewer, longer windows (64 x 64 to 1, CDF 9/7: 11.0 / 10.2 us
// forward / inverse against 17.0 / 15.8 us with 1024 threads and windows
// of 8 pairs; 256 or 128 threads, or 1- or 4-pair windows, are slower).
constexpr int kThreads = 512;
constexpr int kWindowPairs = 2;

struct CtaSync {
    __device__ void operator()() const { __syncthreads(); }
};

// Global -> shared copy of the w x h band: each thread issues kLoadBatch
// loads before their shared-memory stores (a 128 x 128 band crosses the
// L2 once per thread), the flat walk replayed for the stores.
constexpr int kLoadBatch = 16;
__device__ __forceinline__ void load_band(float *A, int P, const float *__restrict__ in, long long in_pitch, int w,
                                          int h)
{
    const int dy = kThreads / w, dx = kThreads - dy * w;
    int y = threadIdx.x / w, x = threadIdx.x - y * w;
    auto advance = [&]() {
        x += dx;
        y += dy;
        if (x >= w) {
            x -= w;
            ++y;
        }
    };
    while (y < h) {
        const int y0 = y, x0 = x;
        float v[kLoadBatch];
#pragma unroll
        for (int k = 0; k < kLoadBatch; ++k) {
            if (y < h) v[k] = __ldg(in + y * in_pitch + x);
            advance();
        }
        y = y0;
        x = x0;
#pragma unroll
        for (int k = 0; k < kLoadBatch; ++k) {
            if (y < h) A[y * P + x] = v[k];
            advance();
        }
    }
}

template <int NS>
__global__ void __launch_bounds__(kThreads)
coarse_forward_kernel(const float *in, long long in_pitch, int w0, int h0, int levels, float *out,
                      long long out_pitch, const Wavelet W)
{
    extern __shared__ __align__(16) float sm[];
    const int P = recur::band_pitch(w0);
    float *A = sm, *B = sm + P * h0;
    pdl_release();
    pdl_wait();
    load_band(A, P, in, in_pitch, w0, h0);
    __syncthreads();
    recur::band_forward<NS, kWindowPairs>(A, B, w0, h0, levels, out, out_pitch, W, threadIdx.x, kThreads, CtaSync{});
}

template <int NS>
__global__ void __launch_bounds__(kThreads)
coarse_inverse_kernel(const float *in, long long in_pitch, int w0, int h0, int levels, float *out,
                      long long out_pitch, const Wavelet W)
{
    extern __shared__ __align__(16) float sm[];
    const int P = recur::band_pitch(w0);
    float *A = sm, *B = sm + P * h0;
    pdl_release();
    pdl_wait();
    load_band(A, P, in, in_pitch, w0, h0);
    __syncthreads();
    recur::band_inverse<NS, kWindowPairs>(A, B, w0, h0, levels, W, threadIdx.x, kThreads, CtaSync{});
    recur::copy_rect(A, P, out, out_pitch, 0, w0, 0, h0, threadIdx.x, kThreads);
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
    // once per process, safe from several host threads
    static const cudaError_t configured = [] {
        cudaError_t e = configure(coarse_forward_kernel<4>);
        if (e == cudaSuccess) e = configure(coarse_inverse_kernel<4>);
        if (e == cudaSuccess) e = configure(coarse_forward_kernel<2>);
        if (e == cudaSuccess) e = configure(coarse_inverse_kernel<2>);
        return e;
    }();
    if (configured != cudaSuccess) return configured;
    if (!coarse_fits(w, h)) return cudaErrorInvalidValue;
    const Wavelet W = make_wavelet(wavelet, inverse);
    const size_t smem = size_t(4) * recur::band_floats(w, h);
    if (wavelet == CDF97) {
        if (inverse)
            return launch_pdl(coarse_inverse_kernel<4>, dim3(1), dim3(kThreads), smem, s, in, in_pitch, w, h, levels, out,
                              out_pitch, W);
        else
            return launch_pdl(coarse_forward_kernel<4>, dim3(1), dim3(kThreads), smem, s, in, in_pitch, w, h, levels, out,
                              out_pitch, W);
    } else {
        if (inverse)
            return launch_pdl(coarse_inverse_kernel<2>, dim3(1), dim3(kThreads), smem, s, in, in_pitch, w, h, levels, out,
                              out_pitch, W);
        else
            return launch_pdl(coarse_forward_kernel<2>, dim3(1), dim3(kThreads), smem, s, in, in_pitch, w, h, levels, out,
                              out_pitch, W);
    }
}

}  // namespace dwt
