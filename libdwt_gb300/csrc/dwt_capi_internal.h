// Host-side internals shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "dwt_pool.h"

namespace dwt {

enum class MemKind { Pageable, Pinned, Device, Managed };

// One GPU context per process: device, working stream of the drop-in calls,
// the buffer pool and the device error word.
struct Context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t s_in = nullptr, s_out = nullptr;  // copy streams of the pipelined host path
    std::vector<cudaEvent_t> events;                 // copy and band events of the pipelined host path
    int *d_err = nullptr;
    Pool pool;
    std::mutex call_mu;  // drop-in calls share `stream`

    // Event i of the pool (created on first use; timing disabled).  Callers
    // hold call_mu.
    cudaEvent_t event(size_t i)
    {
        while (events.size() <= i) {
            cudaEvent_t e = nullptr;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
            events.push_back(e);
        }
        return events[i];
    }
};

Context &ctx();
void ctx_finish();
void log_error(const char *fmt, ...);
int set_error(int code);
MemKind classify(const void *p);
int ceil_log2_int(int x);

// Scratch floats the dense pipelines need for a W x H image over J levels.
size_t dense_scratch_floats(int W, int H, int J, long long *pitch0, long long *pitch1);

// Multi-level dense transforms, out of place, enqueued on `s`.  `in` rows must
// be 16-byte aligned; `out` may be any 4-byte aligned frame.  seg_hint <= 0
// lets the planner pick the row-segment length.
cudaError_t dense_forward(const float *in, long long in_pitch, float *out, long long out_pitch, int W, int H,
                          int J, int wavelet, float *scratch, cudaStream_t s, int *err, int seg_hint);
cudaError_t dense_inverse(const float *in, long long in_pitch, float *out, long long out_pitch, int W, int H,
                          int J, int wavelet, float *scratch, cudaStream_t s, int *err, int seg_hint);

}  // namespace dwt
