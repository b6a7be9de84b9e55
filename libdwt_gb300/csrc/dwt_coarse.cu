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
#include "dwt_lines.cuh"

#include <algorithm>

namespace dwt {

namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
// A: the band, row-major with pitch P; B: its transpose, pitch PT.
template <int NS>
__global__ void __launch_bounds__(kThreads)
coarse_forward_kernel(const float *in, long long in_pitch, int w0, int h0, int levels, float *out,
                      long long out_pitch, const Wavelet W)
{
    extern __shared__ __align__(16) float sm[];
    const int P = coarse_pitch(w0), PT = coarse_pitch(h0);
    float *A = sm, *B = sm + P * h0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int y = threadIdx.x >> 5; y < h0; y += kWarps)
        for (int x = threadIdx.x & 31; x < w0; x += 32) A[y * P + x] = in[y * in_pitch + x];
    __syncthreads();
    int w = w0, h = h0;
    for (int lvl = 0; lvl < levels; ++lvl) {
        const int wd = (w + 1) >> 1, hd = (h + 1) >> 1;
        lines::pass_forward<NS>(A, P, B, PT, h, w, W, warp, kWarps, lane);  // rows -> columns of B
        __syncthreads();
        lines::pass_forward<NS>(B, PT, A, P, w, h, W, warp, kWarps, lane);  // columns -> rows of A
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
    extern __shared__ __align__(16) float sm[];
    const int P = coarse_pitch(w0), PT = coarse_pitch(h0);
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
        lines::pass_inverse<NS>(A, P, B, PT, h, w, W, warp, kWarps, lane);
        __syncthreads();
        // then columns: columns of B hold the L rows then the H rows
        lines::pass_inverse<NS>(B, PT, A, P, w, h, W, warp, kWarps, lane);
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
    const size_t smem = size_t(4) * (coarse_pitch(w) * h + coarse_pitch(h) * w);
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
