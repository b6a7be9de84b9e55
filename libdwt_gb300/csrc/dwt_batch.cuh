// Internal interface of the batched persistent kernel, shared by the batch
// plans (dwt_batch.cu) and the serving loop (dwt_serve.cu).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "../../include/libdwt.h"
#include "dwt_level2d.cuh"

namespace dwt {

constexpr int kMaxLevels = 16;
constexpr int kPhases = kMaxLevels + 1;
constexpr int kBatchWarps = 4;  // warps per CTA (the per-level kernel's shape)

struct BatchImage {
    const float *src;
    long long src_pitch;  // floats, rows 16-byte aligned
    float *dst;
    long long dst_pitch;  // floats
    float *ll[2];         // LL scratch frames (ping-pong)
    long long llp[2];
    int w, h, J, wavelet, inverse;
    int j_tail;  // first level run by the tail item (== J: no tail)
    int seg[kMaxLevels], n_strips[kMaxLevels], n_segs[kMaxLevels];  // per level j (0-based)
    int units[kPhases];  // items per phase
};

struct BatchItem {
    int image;
    int phase;
    int level;  // level index j (forward: j -> j+1; inverse: j -> j-1), -1 for the tail
    int unit;   // strip + seg * n_strips
};

// Fills the descriptor of image `index` (everything but the scratch
// pointers) from the caller's description and the tunables, and appends its
// work items to by_phase[phase].  Returns the scratch floats it needs (0 for
// an image with no levels, which the caller copies as is).
size_t plan_image(BatchImage &I, const dwt_gpu_batch_image &u, const dwt_gpu_batch_params &P, int index,
                  std::vector<std::vector<BatchItem>> &by_phase);

// Points the descriptor's two LL scratch frames into `scratch`.
void set_image_scratch(BatchImage &I, float *scratch);

// Orders the items of every phase by kernel variant (wavelet, direction),
// keeping the image order within a variant, so that the warps of an SM
// mostly run one variant's code at a time (DWT_GPU_BATCH_GROUP_VARIANTS=0:
// no change).  The dependencies are on earlier phases only.
void group_items_by_variant(std::vector<std::vector<BatchItem>> &by_phase, const std::vector<BatchImage> &imgs);

// Shared memory of the batched kernel per CTA.
int batch_smem_bytes();

// Launches the persistent kernel over n_items items (ordered by phase);
// counters: [0] ticket, then kPhases done counters per image, zeroed.
cudaError_t launch_batch_kernel(int grid, const BatchImage *imgs, const BatchItem *items, int n_items,
                                int *counters, int *err, cudaStream_t s);

}  // namespace dwt
