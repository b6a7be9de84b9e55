// dwt_gpu_2_dev_noalloc: the device-resident 2D transform for callers that
// must not allocate device memory.
//
// Who needs it: code that runs where the process's device memory belongs to
// someone else -- a plugin inside a host application whose own allocator is
// the only one allowed to call cudaMalloc, a service that accounts for every
// byte against a fixed budget -- and latency-critical loops that cannot
// afford cudaMalloc / cudaFree, which may synchronize the whole device and
// take unbounded time.  The regular dwt_gpu_2_dev borrows its scratch from the
// library's pool, which grows with cudaMalloc on demand; this variant never
// does.
//
// How: the scratch the transform needs between levels (the LL band of every
// level but the last, ping-ponged between two compact frames) lives in a
// file-scope __device__ array of fixed size, and so does the device error
// word.  Every GPU that loads the library holds that array (about 5.2 MB)
// until the process exits.  Its device address is looked up once per device
// with cudaGetSymbolAddress, on the first call made with that device current;
// make that first call before any stream capture starts.  The caller still
// passes the input and output frames.
//
// Limits and sharing: an image fits when the scratch it needs is at most
// kNoAllocScratchFloats floats -- every image of at most 2048 x 2048 pixels
// does; larger ones are rejected with DWT_GPU_EINVAL before anything is
// enqueued.  All calls share the one array and it keeps whatever the last
// call left in it: every level writes its LL band completely before the next
// level reads it, so nothing in it has to start at zero; the error word does
// and is cleared (stream-ordered) by every call.  Calls whose work overlaps
// on the GPU -- on different streams, or from different host threads without
// ordering between their streams -- race on the array and corrupt each
// other's results.
//
// Errors: arguments are checked before anything is enqueued (overlapping
// source and destination frames included: the level kernels work out of
// place).  A bounded device-side wait that gives up sets the error word;
// dwt_gpu_sync_check reads and clears it (for every device this entry point
// ran on) without creating the library's pooled context.  The device
// addresses are cached per device for the life of the process: a
// cudaDeviceReset invalidates them, and no call may follow one.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/libdwt.h"
#include "dwt_capi_internal.h"
#include "dwt_common.cuh"

namespace dwt {

// LL1 of a 2048 x 2048 image (1024 x 1024, pitch 1024) plus LL2 (512 x 512)
// plus the two 64-float guards the pipeline leaves after each frame.
constexpr size_t kNoAllocScratchFloats = 1024u * 1024u + 512u * 512u + 256u;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float g_noalloc_scratch[kNoAllocScratchFloats];
static __device__ __align__(256) int g_noalloc_err[64];

namespace {

std::mutex g_setup_mu;
float *g_scratch_addr[kMaxDevices] = {};
int *g_err_addr[kMaxDevices] = {};

// Device addresses of the two arrays on the current device (looked up once).
cudaError_t noalloc_addresses(float **scratch, int **err)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void *s = nullptr, *r = nullptr;
        e = cudaGetSymbolAddress(&s, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        e = cudaGetSymbolAddress(&r, g_noalloc_err);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<float *>(s);
        g_err_addr[dev] = static_cast<int *>(r);
    }
    *scratch = g_scratch_addr[dev];
    *err = g_err_addr[dev];
    return cudaSuccess;
}

}  // namespace

int noalloc_device_error()
{
    // every device this entry point has run on: its word is read and cleared
    // with that device current (the caller synchronised the devices)
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) return DWT_GPU_ECUDA;
    int rc = DWT_GPU_OK;
    std::lock_guard<std::mutex> g(g_setup_mu);
    for (int dev = 0; dev < kMaxDevices; ++dev) {
        if (!g_err_addr[dev]) continue;
        int h = 0;
        if (cudaSetDevice(dev) != cudaSuccess ||
            cudaMemcpy(&h, g_err_addr[dev], sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = DWT_GPU_ECUDA;
            continue;
        }
        if (h) {
            cudaMemset(g_err_addr[dev], 0, sizeof(int));
            log_error("dwt_gpu_2_dev_noalloc: device-side wait gave up on device %d (code %d)\n", dev, h);
            if (rc == DWT_GPU_OK) rc = DWT_GPU_EDEVICE;
        }
    }
    cudaSetDevice(cur);
    return rc;
}

}  // namespace dwt

using namespace dwt;

extern "C" int dwt_gpu_2_dev_noalloc(int wavelet, int inverse, const float *src, long long src_pitch_bytes,
                                     float *dst, long long dst_pitch_bytes, int w, int h, int j_levels,
                                     int decompose_one, void *stream)
{
    set_error(DWT_GPU_OK);
    if ((wavelet != CDF97 && wavelet != CDF53) || w <= 0 || h <= 0 || !src || !dst ||
        (src_pitch_bytes % 16) != 0 || (reinterpret_cast<uintptr_t>(src) & 15) != 0 ||
        (dst_pitch_bytes % 4) != 0 || src_pitch_bytes < 4LL * w || dst_pitch_bytes < 4LL * w) {
        log_error("dwt_gpu_2_dev_noalloc: invalid arguments\n");
        return set_error(DWT_GPU_EINVAL);
    }
    const int lim = ceil_log2_int(decompose_one ? (w > h ? w : h) : (w < h ? w : h));
    const int J = (j_levels < 0 || j_levels > lim) ? lim : j_levels;
    long long p0, p1;
    const size_t need = dense_scratch_floats(w, h, J, &p0, &p1);
    if (need > kNoAllocScratchFloats) {
        log_error("dwt_gpu_2_dev_noalloc: a %d x %d image over %d levels needs %zu scratch floats, "
                  "the fixed array holds %zu (images up to 2048 x 2048 fit)\n",
                  w, h, J, need, kNoAllocScratchFloats);
        return set_error(DWT_GPU_EINVAL);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (J == 0) {
        if (src != dst &&
            cudaMemcpy2DAsync(dst, dst_pitch_bytes, src, src_pitch_bytes, size_t(w) * 4, h,
                              cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return set_error(DWT_GPU_ECUDA);
        return 0;
    }
    if (frames_overlap(src, src_pitch_bytes, dst, dst_pitch_bytes, w, h)) {
        log_error("dwt_gpu_2_dev_noalloc: the source and destination frames overlap (out of place only)\n");
        return set_error(DWT_GPU_EINVAL);
    }
    float *scratch = nullptr;
    int *err = nullptr;
    cudaError_t e = noalloc_addresses(&scratch, &err);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), s);
    if (e == cudaSuccess)
        e = inverse ? dense_inverse(src, src_pitch_bytes / 4, dst, dst_pitch_bytes / 4, w, h, J, wavelet,
                                    scratch, s, err, 0)
                    : dense_forward(src, src_pitch_bytes / 4, dst, dst_pitch_bytes / 4, w, h, J, wavelet,
                                    scratch, s, err, 0);
    if (e != cudaSuccess) {
        log_error("dwt_gpu_2_dev_noalloc: CUDA error %s\n", cudaGetErrorString(e));
        return set_error(DWT_GPU_ECUDA);
    }
    set_error(DWT_GPU_OK);
    return J;
}

extern "C" int dwt_gpu_selftest_noalloc_wait_timeout(int iterations)
{
    set_error(DWT_GPU_OK);
    if (iterations <= 0) return set_error(DWT_GPU_EINVAL);
    float *scratch = nullptr;
    int *err = nullptr;
    cudaError_t e = noalloc_addresses(&scratch, &err);
    if (e == cudaSuccess) e = launch_wait_timeout(uint32_t(iterations), err, nullptr);
    if (e != cudaSuccess) {
        log_error("dwt_gpu_selftest_noalloc_wait_timeout: CUDA error %s\n", cudaGetErrorString(e));
        return set_error(DWT_GPU_ECUDA);
    }
    return DWT_GPU_OK;
}
