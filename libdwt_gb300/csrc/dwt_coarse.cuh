// Single-CTA kernel for the coarse levels (see dwt_coarse.cu).
#pragma once

#include "dwt_common.cuh"
#include "dwt_recur.cuh"

namespace dwt {

// Shared memory of the coarse kernel: the band and its half-transformed
// copy, row-major with an odd pitch.
constexpr int kCoarseSmem = 200 * 1024;
// Bands the coarse kernel takes: both buffers within kCoarseSmem.
__host__ __device__ inline bool coarse_fits(int w, int h)
{
    return w >= 1 && h >= 1 && 4LL * recur::band_floats(w, h) <= kCoarseSmem;
}

// Forward: `in` is the w x h LL band entering level j0; runs `levels` levels
// and writes every detail band plus the final LL into the w x h top-left
// region of `out` (the reference layout).  Inverse: `in` is that region of
// the coefficient frame; writes the reconstructed w x h band to `out`.
cudaError_t launch_coarse(bool inverse, const float *in, long long in_pitch, int w, int h, int levels,
                          float *out, long long out_pitch, int wavelet, cudaStream_t s);

}  // namespace dwt
