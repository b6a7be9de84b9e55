// Host-side internals shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <cstdio>
#include <mutex>
#include <vector>

#include "dwt_pool.h"

namespace dwt {

enum class MemKind { Pageable, Pinned, Device, Managed };

// The streams, events and device error word of one drop-in call at a time.
// Calls from several host threads take different lanes, so their copies and
// kernels overlap on the GPU.
struct Lane {
    std::mutex mu;
    int sm_count = 0;
    cudaStream_t stream = nullptr;                  // kernels
    cudaStream_t s_in = nullptr, s_out = nullptr;  // copies of the pipelined host path
    std::vector<cudaEvent_t> events;                 // copy and band events of the pipelined host path
    int *d_err = nullptr;
    int *h_err = nullptr;  // pinned host copy of d_err, read after the stream's synchronisation

    // Event i of the lane (created on first use; timing disabled).  The
    // caller holds mu.
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
constexpr int kCallLanes = 8;

// One GPU context per process: device, the drop-in lanes, the stream and
// device error word of the batched, serving and device-resident forms, and
// the buffer pool.
struct Context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    int *d_err = nullptr;
    Pool pool;
    Lane lanes[kCallLanes];
};

Context &ctx();
void ctx_finish();

// A named range on the calling thread for the duration of a scope, shown
// by Nsight Systems on the timeline (free when no tool is attached).
class NvtxRange {
public:
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    template <typename... A>
    NvtxRange(const char *fmt, A... args)
    {
        char buf[96];
        snprintf(buf, sizeof buf, fmt, args...);
        nvtxRangePushA(buf);
    }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Holds a drop-in lane for the duration of a call: a free one if any, else
// the calling thread's own (waiting for it).
class LaneGuard {
public:
    explicit LaneGuard(Context &c);
    ~LaneGuard() { lane_->mu.unlock(); }
    LaneGuard(const LaneGuard &) = delete;
    LaneGuard &operator=(const LaneGuard &) = delete;
    Lane &get() { return *lane_; }

private:
    Lane *lane_;
};
void log_error(const char *fmt, ...);
int set_error(int code);
MemKind classify(const void *p);
int ceil_log2_int(int x);

// Whether the byte spans of two w x h float frames (first sample to last
// sample of the last row) intersect.  The out-of-place device forms refuse
// such pairs: a level kernel would read samples another tile already wrote.
inline bool frames_overlap(const void *a, long long a_pitch_bytes, const void *b, long long b_pitch_bytes, int w,
                           int h)
{
    const unsigned long long a0 = reinterpret_cast<uintptr_t>(a), b0 = reinterpret_cast<uintptr_t>(b);
    const unsigned long long a1 = a0 + (unsigned long long)(h - 1) * a_pitch_bytes + 4ull * w;
    const unsigned long long b1 = b0 + (unsigned long long)(h - 1) * b_pitch_bytes + 4ull * w;
    return a0 < b1 && b0 < a1;
}

// Reads and clears the error word of the allocation-free entry point on every
// device it ran on (DWT_GPU_OK when it never ran, DWT_GPU_EDEVICE when a
// device-side wait of it gave up); the caller has synchronised the devices.
int noalloc_device_error();

// Enqueues a one-warp kernel whose bounded mbarrier wait is never satisfied:
// it gives up after `iterations` tries and sets *err (no fault).
cudaError_t launch_wait_timeout(uint32_t iterations, int *err, cudaStream_t s);

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
