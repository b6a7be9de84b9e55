// All remaining coarse levels of one image in a single CTA.
//
// Once the LL band is small (at most kCoarseMax samples), each further level
// has too little work to fill the GPU and a launch per level costs more than
// the level itself.  This kernel loads the band into shared memory and runs
// every remaining level there: per level a row pass and a column pass, each
// as parallel lifting sweeps (one __syncthreads per sweep) with the same
// per-sample arithmetic as the reference (x + c*(l + r), symmetric
// extension, scaling), then deinterleaves into the second buffer.  The
// forward writes each level's detail bands and the final LL to the output
// frame; the inverse reads them and writes the reconstructed band.
#include "dwt_coarse.cuh"

#include <algorithm>

namespace dwt {

namespace {

constexpr int kThreads = 1024;

// One lifting step on samples of `parity` of `nl` lines of length n:
// line l, sample i at buf[l*ls + i*es].  Consecutive threads take
// consecutive lines when lines are adjacent in memory (ls == 1, the column
// pass) and consecutive samples otherwise, so shared-memory accesses of a
// warp spread over the banks.
__device__ __forceinline__ void sweep(float *buf, int ls, int es, int nl, int n, int parity, float c)
{
    const int half = (n - parity + 1) >> 1;  // samples of this parity
    const int tot = nl * half;
    for (int k = threadIdx.x; k < tot; k += blockDim.x) {
        int l, j;
        if (ls == 1) {
            j = k / nl;
            l = k - j * nl;
        } else {
            l = k / half;
            j = k - l * half;
        }
        const int i = parity + 2 * j;
        float *x = buf + l * ls;
        const float left = (i > 0) ? x[(i - 1) * es] : x[(i + 1) * es];
        const float right = (i + 1 < n) ? x[(i + 1) * es] : x[(i - 1) * es];
        x[i * es] = lift(x[i * es], c, left, right);
    }
}

// Forward lifting of nl lines of length n >= 2 in place (no scaling).
__device__ __forceinline__ void lines_lift_fwd(float *buf, int ls, int es, int nl, int n, const Wavelet &W)
{
    for (int s = 0; s < W.nsteps; ++s) {
        sweep(buf, ls, es, nl, n, (s & 1) ? 0 : 1, W.c[s]);
        __syncthreads();
    }
}

__device__ __forceinline__ void lines_lift_inv(float *buf, int ls, int es, int nl, int n, const Wavelet &W)
{
    for (int s = 0; s < W.nsteps; ++s) {
        sweep(buf, ls, es, nl, n, (s & 1) ? 1 : 0, W.c[s]);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kThreads)
coarse_forward_kernel(const float *in, long long in_pitch, int w0, int h0, int levels, float *out,
                      long long out_pitch, const Wavelet W)
{
    extern __shared__ float sm[];
    const int P = w0;
    float *A = sm, *B = sm + P * h0;
    for (int k = threadIdx.x; k < w0 * h0; k += blockDim.x) {
        const int y = k / w0, x = k - y * w0;
        A[y * P + x] = in[y * in_pitch + x];
    }
    __syncthreads();
    int w = w0, h = h0;
    for (int lvl = 0; lvl < levels; ++lvl) {
        const int wd = (w + 1) >> 1, hd = (h + 1) >> 1;
        // rows y < h, length w: lift in A, then scale + deinterleave into B
        if (w > 1) lines_lift_fwd(A, P, 1, h, w, W);
        for (int k = threadIdx.x; k < w * h; k += blockDim.x) {
            const int y = k / w, x = k - y * w;
            const float v = A[y * P + x];
            if (w == 1)
                B[y * P] = fmul(v, W.n1_fwd);
            else if ((x & 1) == 0)
                B[y * P + (x >> 1)] = fmul(v, W.zeta_e);
            else
                B[y * P + wd + (x >> 1)] = fmul(v, W.zeta_o);
        }
        __syncthreads();
        // columns x < w, length h: lift in B, then scale + deinterleave into A
        if (h > 1) lines_lift_fwd(B, 1, P, w, h, W);
        for (int k = threadIdx.x; k < w * h; k += blockDim.x) {
            const int y = k / w, x = k - y * w;
            const float v = B[y * P + x];
            if (h == 1)
                A[x] = fmul(v, W.n1_fwd);
            else if ((y & 1) == 0)
                A[(y >> 1) * P + x] = fmul(v, W.zeta_e);
            else
                A[(hd + (y >> 1)) * P + x] = fmul(v, W.zeta_o);
        }
        __syncthreads();
        // this level's detail bands are final
        for (int k = threadIdx.x; k < w * h; k += blockDim.x) {
            const int y = k / w, x = k - y * w;
            if (x >= wd || y >= hd) out[y * out_pitch + x] = A[y * P + x];
        }
        w = wd;
        h = hd;
    }
    for (int k = threadIdx.x; k < w * h; k += blockDim.x) {
        const int y = k / w, x = k - y * w;
        out[y * out_pitch + x] = A[y * P + x];
    }
}

__global__ void __launch_bounds__(kThreads)
coarse_inverse_kernel(const float *in, long long in_pitch, int w0, int h0, int levels, float *out,
                      long long out_pitch, const Wavelet W)
{
    extern __shared__ float sm[];
    const int P = w0;
    float *A = sm, *B = sm + P * h0;
    for (int k = threadIdx.x; k < w0 * h0; k += blockDim.x) {
        const int y = k / w0, x = k - y * w0;
        A[y * P + x] = in[y * in_pitch + x];
    }
    __syncthreads();
    for (int lvl = levels - 1; lvl >= 0; --lvl) {
        int w = w0, h = h0;
        for (int k = 0; k < lvl; ++k) {
            w = (w + 1) >> 1;
            h = (h + 1) >> 1;
        }
        const int ws = (w + 1) >> 1, hs = (h + 1) >> 1;
        // rows y < h: interleave L (cols < ws) and H (cols >= ws) into B with
        // the pre-scaling, then lift (src/libdwt.c:5806-5811)
        for (int k = threadIdx.x; k < w * h; k += blockDim.x) {
            const int y = k / w, x = k - y * w;
            if (w == 1)
                B[y * P] = fmul(A[y * P], W.n1_inv);
            else if ((x & 1) == 0)
                B[y * P + x] = fmul(A[y * P + (x >> 1)], W.zeta_o);
            else
                B[y * P + x] = fmul(A[y * P + ws + (x >> 1)], W.zeta_e);
        }
        __syncthreads();
        if (w > 1) lines_lift_inv(B, P, 1, h, w, W);
        // columns x < w: interleave L rows and H rows into A, pre-scale, lift
        for (int k = threadIdx.x; k < w * h; k += blockDim.x) {
            const int y = k / w, x = k - y * w;
            if (h == 1)
                A[x] = fmul(B[x], W.n1_inv);
            else if ((y & 1) == 0)
                A[y * P + x] = fmul(B[(y >> 1) * P + x], W.zeta_o);
            else
                A[y * P + x] = fmul(B[(hs + (y >> 1)) * P + x], W.zeta_e);
        }
        __syncthreads();
        if (h > 1) lines_lift_inv(A, 1, P, w, h, W);
    }
    for (int k = threadIdx.x; k < w0 * h0; k += blockDim.x) {
        const int y = k / w0, x = k - y * w0;
        out[y * out_pitch + x] = A[y * P + x];
    }
}

template <typename K>
cudaError_t configure(K kernel)
{
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                2 * kCoarseMax * 4);
}

}  // namespace

cudaError_t launch_coarse(bool inverse, const float *in, long long in_pitch, int w, int h, int levels,
                          float *out, long long out_pitch, int wavelet, cudaStream_t s)
{
    static bool configured = false;
    if (!configured) {
        cudaError_t e = configure(coarse_forward_kernel);
        if (e == cudaSuccess) e = configure(coarse_inverse_kernel);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    if ((long long)w * h > kCoarseMax || w <= 0 || h <= 0) return cudaErrorInvalidValue;
    const Wavelet W = make_wavelet(wavelet, inverse);
    const size_t smem = size_t(2) * w * h * 4;
    if (inverse)
        coarse_inverse_kernel<<<1, kThreads, smem, s>>>(in, in_pitch, w, h, levels, out, out_pitch, W);
    else
        coarse_forward_kernel<<<1, kThreads, smem, s>>>(in, in_pitch, w, h, levels, out, out_pitch, W);
    return cudaGetLastError();
}

}  // namespace dwt
