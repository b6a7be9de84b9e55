// Banks of interleaved 1D signals, transformed in place in one launch.
//
// The layout of a caller that runs dwt_cdf97_{f,i}_ex_stride_s over many
// signals stored G to a group, sample-interleaved (sample i of signal s of
// group g at g*group_stride + (i*G + s)*4 bytes), with L written to samples
// [0, ceil(N/2)) and H to [ceil(N/2), N) of each signal.  One CTA owns one
// group: it copies the group's N*G floats into shared memory with vector
// loads, then every thread runs the lifting recurrence down a segment of one
// signal (warmed up by the lifting latency) reading the staged samples, and
// writes its finished L and H samples straight back to global memory.  All
// of a group's samples are read before any is written, so in place is safe,
// and each sample crosses HBM once each way (8 bytes per sample).
#include "dwt_signals.cuh"
#include "dwt_recur.cuh"

#include <algorithm>

namespace dwt {

namespace {

constexpr int kSigThreads = 512;
constexpr uint32_t kBulkChunk = 32768;  // bytes per bulk copy

template <int NS, bool INV>
__global__ void __launch_bounds__(kSigThreads)
signals_kernel(float *base, int N, int G, long long group_stride_f, long long groups, int seg, const Wavelet W,
               int *err)
{
    extern __shared__ __align__(128) float sx[];
    __shared__ __align__(8) uint64_t bar;
    const uint32_t bytes = uint32_t(N) * uint32_t(G) * 4u;  // a multiple of 16
    const int per_signal = kSigThreads / G;
    const int s = threadIdx.x % G, c = threadIdx.x / G;
    const int npairs = (N + 1) >> 1;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t phase = 0;
    // the TMA engine stages the whole group block; one mbarrier phase per group
    auto stage = [&](long long g) {
        const char *src = reinterpret_cast<const char *>(base + g * group_stride_f);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bar, bytes);
        for (uint32_t o = 0; o < bytes; o += kBulkChunk)
            bulk_g2s(reinterpret_cast<char *>(sx) + o, src + o, min(kBulkChunk, bytes - o), &bar);
    };
    if (threadIdx.x == 0 && blockIdx.x < groups) stage(blockIdx.x);
    for (long long g = blockIdx.x; g < groups; g += gridDim.x) {
        float *gb = base + g * group_stride_f;
        if (!mbar_wait_bounded(&bar, phase)) {
            if (threadIdx.x == 0) atomicCAS(err, 0, kErrWaitTimeout);
            return;
        }
        phase ^= 1u;
        if (N == 1) {
            if (c == 0) gb[s] = fmul(sx[s], INV ? W.n1_inv : W.n1_fwd);
        } else {
            for (int k0 = c * seg; k0 < npairs; k0 += per_signal * seg) {
                const int k1 = min(k0 + seg, npairs);
                if (INV)
                    recur::line_inverse<NS>(sx + s, G, N, gb + s, G, k0, k1, W);
                else
                    recur::line_forward<NS>(sx + s, G, N, gb + s, G, k0, k1, W);
            }
        }
        __syncthreads();  // every thread is done with the staged block
        if (threadIdx.x == 0 && g + gridDim.x < groups) stage(g + gridDim.x);
    }
}

template <int NS, bool INV>
cudaError_t launch_t(float *base, int N, int G, long long group_stride_f, long long groups, cudaStream_t s,
                     int sm_count, int *err)
{
    const size_t smem = size_t(N) * G * 4;
    // once per instantiation, safe from several host threads
    static const cudaError_t configured =
        cudaFuncSetAttribute(signals_kernel<NS, INV>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSignalsMaxSmem);
    if (configured != cudaSuccess) return configured;
    const int per_signal = kSigThreads / G;
    const int npairs = (N + 1) / 2;
    const int seg = (npairs + per_signal - 1) / per_signal;
    const int per_sm = int(std::max<size_t>(1, size_t(kSignalsMaxSmem) / std::max<size_t>(smem, 1)));
    const long long grid = std::min<long long>(groups, (long long)sm_count * std::min(per_sm, 8));
    const Wavelet W = make_wavelet(NS == 4 ? CDF97 : CDF53, INV);
    signals_kernel<NS, INV><<<int(grid), kSigThreads, smem, s>>>(base, N, G, group_stride_f, groups, seg, W, err);
    return cudaGetLastError();
}

}  // namespace

bool signals_fast_ok(const void *base, int N, long long stride, int G, long long group_stride, long long lane_stride)
{
    if (N <= 0 || G <= 0 || kSigThreads % G != 0) return false;
    if (lane_stride != 4 || stride != 4LL * G) return false;
    if ((4LL * N * G) % 16 != 0 || (long long)N * G * 4 > kSignalsMaxSmem) return false;
    if ((reinterpret_cast<uintptr_t>(base) & 15) != 0 || group_stride % 16 != 0) return false;
    if (group_stride < 4LL * N * G) return false;
    return true;
}

cudaError_t launch_signals(int wavelet, bool inverse, float *base, int N, int G, long long group_stride_bytes,
                           long long groups, cudaStream_t s, int sm_count, int *err)
{
    const long long gs = group_stride_bytes / 4;
    if (wavelet == CDF97)
        return inverse ? launch_t<4, true>(base, N, G, gs, groups, s, sm_count, err)
                       : launch_t<4, false>(base, N, G, gs, groups, s, sm_count, err);
    return inverse ? launch_t<2, true>(base, N, G, gs, groups, s, sm_count, err)
                   : launch_t<2, false>(base, N, G, gs, groups, s, sm_count, err);
}

}  // namespace dwt
