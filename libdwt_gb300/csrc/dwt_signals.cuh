// In-place transform of banks of sample-interleaved 1D signals (see
// dwt_signals.cu).
#pragma once

#include "dwt_common.cuh"

namespace dwt {

// Shared memory a group block may take (N * G floats).
constexpr int kSignalsMaxSmem = 200 * 1024;

// Whether the bank layout (sample i of signal s of group g at
// g*group_stride + i*stride + (s % G)*lane_stride bytes from base) is the
// dense interleave this kernel takes.
bool signals_fast_ok(const void *base, int N, long long stride, int G, long long group_stride, long long lane_stride);

// One level over `groups` groups of G signals of N samples, in place.
cudaError_t launch_signals(int wavelet, bool inverse, float *base, int N, int G, long long group_stride_bytes,
                           long long groups, cudaStream_t s, int sm_count, int *err);

}  // namespace dwt
