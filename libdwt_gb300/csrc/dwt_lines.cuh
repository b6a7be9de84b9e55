// Line transforms held in a warp's registers (device code shared by the
// coarse-level kernel and the batched kernel's tail items).
//
// A warp holds one line (row or column) of up to 252 samples, 8 per lane,
// samples past the end of the line loaded as their mirror images, and runs
// the lifting steps with warp shuffles: the same per-sample arithmetic as the
// reference (x + c*(l + r), symmetric extension, scaling).  A pass writes its
// lines transposed and deinterleaved into the other buffer, so the next pass
// reads its lines as rows too.
#pragma once

#include "dwt_common.cuh"

namespace dwt {
namespace lines {

constexpr int kV = 8;  // samples per lane: one warp holds 256 samples of a line
constexpr unsigned kAll = 0xffffffffu;

__device__ __forceinline__ bool aligned16(const float *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

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
                                             const Wavelet &W, int warp, int nwarps, int lane)
{
    const int nd = (n + 1) >> 1;
    if (n == 1) {
        for (int l = warp * 32 + lane; l < nl; l += nwarps * 32) dst[l] = fmul(src[l * ls], W.n1_fwd);
        return;
    }
    int ld[kV], st[kV];
#pragma unroll
    for (int k = 0; k < kV; ++k) {
        const int i = kV * lane + k;
        ld[k] = mirror(i, n);
        st[k] = i < n ? ((k & 1) ? nd + (i >> 1) : (i >> 1)) * dp : -1;
    }
    // lanes whose 8 samples lie inside the line read them as two 16-byte
    // loads, when every line starts on a 16-byte boundary
    const bool vec = (kV * lane + kV <= n) && ((ls & 3) == 0) && aligned16(src);
    for (int l = warp; l < nl; l += nwarps) {
        const float *line = src + l * ls;
        float x[kV];
        if (vec) {
            const float4 a = *reinterpret_cast<const float4 *>(line + kV * lane);
            const float4 b = *reinterpret_cast<const float4 *>(line + kV * lane + 4);
            x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
            x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
        } else {
#pragma unroll
            for (int k = 0; k < kV; ++k) x[k] = line[ld[k]];
        }
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
                                             const Wavelet &W, int warp, int nwarps, int lane)
{
    const int nd = (n + 1) >> 1;
    if (n == 1) {
        for (int l = warp * 32 + lane; l < nl; l += nwarps * 32) dst[l] = fmul(src[l * ls], W.n1_inv);
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
    // lanes whose 8 samples lie inside the line read their 4 L and 4 H
    // samples as two 16-byte loads when both halves start 16-byte aligned
    const bool vec = (kV * lane + kV <= n) && ((ls & 3) == 0) && ((nd & 3) == 0) && aligned16(src);
    for (int l = warp; l < nl; l += nwarps) {
        const float *line = src + l * ls;
        float x[kV];
        if (vec) {
            const float4 a = *reinterpret_cast<const float4 *>(line + 4 * lane);
            const float4 b = *reinterpret_cast<const float4 *>(line + nd + 4 * lane);
            x[0] = a.x; x[1] = b.x; x[2] = a.y; x[3] = b.y;
            x[4] = a.z; x[5] = b.z; x[6] = a.w; x[7] = b.w;
        } else {
#pragma unroll
            for (int k = 0; k < kV; ++k) x[k] = line[ld[k]];
        }
        line_inverse<NS>(x, W, lane);
#pragma unroll
        for (int k = 0; k < kV; ++k)
            if (st[k] >= 0) dst[st[k] + l] = x[k];
    }
}


}  // namespace lines
}  // namespace dwt
