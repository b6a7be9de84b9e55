// Single-CTA kernel for the coarse levels (see dwt_coarse.cu).
#pragma once

#include "dwt_common.cuh"

namespace dwt {

// Largest band (w * h samples) the coarse kernel takes: two float buffers of
// this size live in shared memory.
constexpr int kCoarseMax = 16384;

// Forward: `in` is the w x h LL band entering level j0; runs `levels` levels
// and writes every detail band plus the final LL into the w x h top-left
// region of `out` (the reference layout).  Inverse: `in` is that region of
// the coefficient frame; writes the reconstructed w x h band to `out`.
cudaError_t launch_coarse(bool inverse, const float *in, long long in_pitch, int w, int h, int levels,
                          float *out, long long out_pitch, int wavelet, cudaStream_t s);

}  // namespace dwt
