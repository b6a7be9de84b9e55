// C-ABI of libdwt_gb300: libdwt's own entry points for the lifting hot path
// (src/libdwt.h) plus the dwt_gpu_* extensions, over one GPU context.
//
// Every 2D call runs the same device pipeline:
//   1. stage the caller's frame into a compact device frame IN whose rows are
//      16-byte aligned (cudaMemcpy2DAsync for host memory with 4-byte pixels,
//      a byte-gather kernel for anything else);
//   2. transform IN -> OUT out of place, one fused level kernel per level,
//      coarser LL bands ping-ponging between two compact scratch frames;
//   3. write OUT back in the caller's layout (or have the level kernels write
//      straight into a dense device caller frame).
// Out of place is what makes the fused kernel legal: the reference works in
// place, where one tile's outputs land on other tiles' inputs.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/libdwt.h"
#include "dwt_capi_internal.h"
#include "dwt_coarse.cuh"
#include "dwt_double.cuh"
#include "dwt_generic.cuh"
#include "dwt_signals.cuh"
#include "dwt_level2d.cuh"

namespace dwt {

// ---------------------------------------------------------------- context

static std::mutex g_init_mu;
static Context *g_ctx = nullptr;
static std::atomic<int> g_accel{0};
static thread_local int t_last_error = DWT_GPU_OK;

void log_error(const char *fmt, ...)
{
    // the reference's LOG_ERR format (src/libdwt.c:7953-7985)
    flockfile(stderr);
    fputs("ERROR: ", stderr);
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    va_end(ap);
    fflush(stderr);
    funlockfile(stderr);
}

int set_error(int code)
{
    t_last_error = code;
    return code;
}

Context &ctx()
{
    std::lock_guard<std::mutex> g(g_init_mu);
    if (!g_ctx) {
        Context *c = new Context();
        const char *dev = getenv("DWT_GPU_DEVICE");
        c->device = dev ? atoi(dev) : 0;
        cudaSetDevice(c->device);
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        cudaMalloc(&c->d_err, sizeof(int));
        cudaMemset(c->d_err, 0, sizeof(int));
        cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
        // the copy streams run at the highest priority: where copies are
        // kernels (host memory the GPU addresses itself) their blocks go
        // ahead of the band kernels' queued blocks
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        for (Lane &l : c->lanes) {
            l.sm_count = c->sm_count;
            cudaStreamCreateWithFlags(&l.stream, cudaStreamNonBlocking);
            cudaStreamCreateWithPriority(&l.s_in, cudaStreamNonBlocking, greatest);
            cudaStreamCreateWithPriority(&l.s_out, cudaStreamNonBlocking, greatest);
            cudaMalloc(&l.d_err, sizeof(int));
            cudaMemset(l.d_err, 0, sizeof(int));
            if (cudaHostAlloc(reinterpret_cast<void **>(&l.h_err), sizeof(int), cudaHostAllocDefault) != cudaSuccess) {
                l.h_err = nullptr;
                cudaGetLastError();
            }
        }
        cudaDeviceSynchronize();
        g_ctx = c;
    }
    cudaSetDevice(g_ctx->device);
    return *g_ctx;
}

void ctx_finish()
{
    std::lock_guard<std::mutex> g(g_init_mu);
    if (!g_ctx) return;
    cudaStreamSynchronize(g_ctx->stream);
    for (Lane &l : g_ctx->lanes) {
        std::lock_guard<std::mutex> lg(l.mu);
        cudaStreamSynchronize(l.stream);
    }
    g_ctx->pool.release_all();
    cudaFree(g_ctx->d_err);
    for (Lane &l : g_ctx->lanes) {
        for (cudaEvent_t e : l.events) cudaEventDestroy(e);
        cudaStreamDestroy(l.s_in);
        cudaStreamDestroy(l.s_out);
        cudaStreamDestroy(l.stream);
        cudaFree(l.d_err);
        if (l.h_err) cudaFreeHost(l.h_err);
        l.h_err = nullptr;
    }
    cudaStreamDestroy(g_ctx->stream);
    delete g_ctx;
    g_ctx = nullptr;
}

LaneGuard::LaneGuard(Context &c)
{
    for (Lane &l : c.lanes)
        if (l.mu.try_lock()) {
            lane_ = &l;
            return;
        }
    lane_ = &c.lanes[std::hash<std::thread::id>{}(std::this_thread::get_id()) % kCallLanes];
    lane_->mu.lock();
}

// ------------------------------------------------------------ helpers

int ceil_log2_int(int x)
{
    int r = 0;
    while ((1LL << r) < (long long)x) r++;
    return r;
}

MemKind classify(const void *p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return MemKind::Pageable;
    }
    switch (a.type) {
    case cudaMemoryTypeDevice: return MemKind::Device;
    case cudaMemoryTypeManaged: return MemKind::Managed;
    case cudaMemoryTypeHost: return MemKind::Pinned;
    default: return MemKind::Pageable;
    }
}

static long long align_up(long long v, long long a) { return (v + a - 1) / a * a; }

// Scoped pool allocation on the context stream.
struct Buf {
    void *p = nullptr;
    cudaStream_t s = nullptr;
    Buf() = default;
    Buf(size_t bytes, cudaStream_t st) { alloc(bytes, st); }
    bool alloc(size_t bytes, cudaStream_t st)
    {
        s = st;
        p = ctx().pool.alloc(bytes, st);
        return p != nullptr;
    }
    ~Buf()
    {
        if (p) ctx().pool.release(p, s);
    }
    Buf(const Buf &) = delete;
    Buf &operator=(const Buf &) = delete;
    float *f() const { return static_cast<float *>(p); }
};

#define CK(x)                                                                  \
    do {                                                                       \
        cudaError_t e_ = (x);                                                  \
        if (e_ != cudaSuccess) {                                               \
            log_error("CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
            return set_error(e_ == cudaErrorMemoryAllocation ? DWT_GPU_ENOMEM : DWT_GPU_ECUDA); \
        }                                                                      \
    } while (0)

// Reads and clears a device error word after its stream drained.
static int check_device_error(int *d_err)
{
    int h = 0;
    if (cudaMemcpy(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return DWT_GPU_ECUDA;
    if (h) {
        cudaMemset(d_err, 0, sizeof(int));
        log_error("device-side wait gave up (code %d)\n", h);
        return DWT_GPU_EDEVICE;
    }
    return DWT_GPU_OK;
}
static int check_device_error(Context &c) { return check_device_error(c.d_err); }
static int check_device_error(Lane &l) { return check_device_error(l.d_err); }

// The end of a call on a lane: waits for the lane's stream and reports (and
// clears) its device error word, which the same stream copies into pinned
// host memory first, so that one synchronisation serves both (a separate
// synchronous copy of the word cost about as much as a small call's work).
static int lane_finish(Lane &l)
{
    if (!l.h_err) {
        if (cudaStreamSynchronize(l.stream) != cudaSuccess) {
            log_error("CUDA error %s\n", cudaGetErrorString(cudaGetLastError()));
            return DWT_GPU_ECUDA;
        }
        return check_device_error(l);
    }
    cudaError_t e = cudaMemcpyAsync(l.h_err, l.d_err, sizeof(int), cudaMemcpyDeviceToHost, l.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(l.stream);
    if (e != cudaSuccess) {
        log_error("CUDA error %s\n", cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? DWT_GPU_ENOMEM : DWT_GPU_ECUDA;
    }
    const int h = *reinterpret_cast<volatile int *>(l.h_err);
    if (h) {
        cudaMemsetAsync(l.d_err, 0, sizeof(int), l.stream);
        cudaStreamSynchronize(l.stream);
        log_error("device-side wait gave up (code %d)\n", h);
        return DWT_GPU_EDEVICE;
    }
    return DWT_GPU_OK;
}

// ------------------------------------------------------- level pipelines

size_t dense_scratch_floats(int W, int H, int J, long long *pitch0, long long *pitch1)
{
    const int w1 = (W + 1) / 2, h1 = (H + 1) / 2, w2 = (W + 3) / 4, h2 = (H + 3) / 4;
    *pitch0 = align_up(w1, 32);
    *pitch1 = align_up(w2, 32);
    size_t n = 0;
    if (J >= 2) n += size_t(*pitch0) * h1 + 64;
    if (J >= 3) n += size_t(*pitch1) * h2 + 64;
    return n;
}

// Largest band (pixels) handed to the single-CTA coarse kernel: a 128 x 128
// band already runs faster as one more level on the whole GPU (16384^2 CDF
// 9/7 forward, full depth: 508 us with the coarse kernel from 64 x 64 on,
// 512-518 us from 128 x 128).
static long long coarse_max_pixels()
{
    static const long long n = [] {
        const char *e = getenv("DWT_GPU_COARSE_PX");
        const long long v = e ? atoll(e) : 0;
        return v > 0 ? v : 4096;
    }();
    return n;
}

// First level whose LL band fits the single-CTA coarse kernel (J if none).
static int coarse_level(int W, int H, int J)
{
    for (int j = 0; j < J; ++j) {
        const int w = ceil_div_pow2(W, j), h = ceil_div_pow2(H, j);
        if (coarse_fits(w, h) && (long long)w * h <= coarse_max_pixels()) return j;
    }
    return J;
}

// Descriptor of forward level j (LL_j -> LL_{j+1} in scratch, or in `out`
// for the last level, and the three detail bands in `out`).
static LevelDesc fwd_desc(const float *in, long long in_pitch, float *out, long long out_pitch, int W, int H,
                          int J, int j, float *const buf[2], const long long p[2])
{
    const int w = ceil_div_pow2(W, j), h = ceil_div_pow2(H, j);
    const int wd = (w + 1) / 2, hd = (h + 1) / 2;
    LevelDesc d{};
    d.w = w;
    d.h = h;
    d.in[0] = j == 0 ? in : buf[(j - 1) % 2];
    d.in_pitch[0] = j == 0 ? in_pitch : p[(j - 1) % 2];
    if (j == J - 1) {
        d.out[0] = out;
        d.out_pitch[0] = out_pitch;
    } else {
        d.out[0] = buf[j % 2];
        d.out_pitch[0] = p[j % 2];
    }
    d.out[1] = out + wd;
    d.out[2] = out + hd * out_pitch;
    d.out[3] = out + hd * out_pitch + wd;
    d.out_pitch[1] = d.out_pitch[2] = d.out_pitch[3] = out_pitch;
    return d;
}

// Descriptor of inverse level j (LL_j and the details of level j -> LL_{j-1}).
static LevelDesc inv_desc(const float *in, long long in_pitch, float *out, long long out_pitch, int W, int H,
                          int J, int j, float *const buf[2], const long long p[2])
{
    const int w = ceil_div_pow2(W, j - 1), h = ceil_div_pow2(H, j - 1);
    const int ws = (w + 1) / 2, hs = (h + 1) / 2;
    LevelDesc d{};
    d.w = w;
    d.h = h;
    d.in[0] = j == J ? in : buf[(j - 1) % 2];
    d.in_pitch[0] = j == J ? in_pitch : p[(j - 1) % 2];
    d.in[1] = in + ws;
    d.in[2] = in + hs * in_pitch;
    d.in[3] = in + hs * in_pitch + ws;
    d.in_pitch[1] = d.in_pitch[2] = d.in_pitch[3] = in_pitch;
    if (j == 1) {
        d.out[0] = out;
        d.out_pitch[0] = out_pitch;
    } else {
        d.out[0] = buf[(j - 2) % 2];
        d.out_pitch[0] = p[(j - 2) % 2];
    }
    return d;
}

static void scratch_frames(int W, int H, int J, float *scratch, float *buf[2], long long p[2])
{
    dense_scratch_floats(W, H, J, &p[0], &p[1]);
    buf[0] = scratch;
    buf[1] = scratch + (J >= 2 ? size_t(p[0]) * ((H + 1) / 2) + 64 : 0);
}

// Consecutive levels hand out their segments in alternate directions, so a
// level starts on the rows of its input band the previous level wrote last,
// some of them still in L2 (16384^2 CDF 9/7: 499.3 / 551.1 us forward /
// inverse against 500.7 / 553.0 us in one direction).
constexpr bool kAlternateOrder = true;

// Forward levels j_begin .. J-1 (the coarse kernel takes over once the band fits).
static cudaError_t dense_forward_levels(const float *in, long long in_pitch, float *out, long long out_pitch,
                                        int W, int H, int J, int j_begin, int wavelet, float *scratch,
                                        cudaStream_t s, int *err, int seg_hint, cudaEvent_t after_first = nullptr)
{
    float *buf[2];
    long long p[2];
    scratch_frames(W, H, J, scratch, buf, p);
    const int j0 = std::max(coarse_level(W, H, J), j_begin);
    for (int j = j_begin; j < j0; ++j) {
        const NvtxRange range("level %d forward %dx%d", j, ceil_div_pow2(W, j), ceil_div_pow2(H, j));
        LevelDesc d = fwd_desc(in, in_pitch, out, out_pitch, W, H, J, j, buf, p);
        plan_level(d, seg_hint, false);
        d.reverse = kAlternateOrder && ((j - j_begin) & 1);
        cudaError_t e = launch_level(d, wavelet, false, s, err);
        if (e == cudaSuccess && after_first && j == j_begin) e = cudaEventRecord(after_first, s);
        if (e != cudaSuccess) return e;
    }
    if (j0 < J) {
        const float *src = j0 == 0 ? in : buf[(j0 - 1) % 2];
        const long long sp = j0 == 0 ? in_pitch : p[(j0 - 1) % 2];
        return launch_coarse(false, src, sp, ceil_div_pow2(W, j0), ceil_div_pow2(H, j0), J - j0, out,
                             out_pitch, wavelet, s);
    }
    return cudaSuccess;
}

// Inverse levels J .. j_end (j_end >= 1).
static cudaError_t dense_inverse_levels(const float *in, long long in_pitch, float *out, long long out_pitch,
                                        int W, int H, int J, int j_end, int wavelet, float *scratch,
                                        cudaStream_t s, int *err, int seg_hint)
{
    float *buf[2];
    long long p[2];
    scratch_frames(W, H, J, scratch, buf, p);
    const int j0 = coarse_level(W, H, J);
    int jtop = J;  // level whose LL the next level kernel reads
    if (j0 < J && j0 >= j_end - 1) {
        float *dst = j0 == 0 ? out : buf[(j0 - 1) % 2];
        const long long dp = j0 == 0 ? out_pitch : p[(j0 - 1) % 2];
        cudaError_t e = launch_coarse(true, in, in_pitch, ceil_div_pow2(W, j0), ceil_div_pow2(H, j0), J - j0,
                                      dst, dp, wavelet, s);
        if (e != cudaSuccess) return e;
        jtop = j0;
    }
    for (int j = jtop; j >= j_end; --j) {
        const NvtxRange range("level %d inverse %dx%d", j - 1, ceil_div_pow2(W, j - 1), ceil_div_pow2(H, j - 1));
        LevelDesc d = inv_desc(in, in_pitch, out, out_pitch, W, H, J, j, buf, p);
        plan_level(d, seg_hint, true);
        d.reverse = kAlternateOrder && ((jtop - j) & 1);
        cudaError_t e = launch_level(d, wavelet, true, s, err);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t dense_forward(const float *in, long long in_pitch, float *out, long long out_pitch, int W, int H,
                          int J, int wavelet, float *scratch, cudaStream_t s, int *err, int seg_hint)
{
    return dense_forward_levels(in, in_pitch, out, out_pitch, W, H, J, 0, wavelet, scratch, s, err, seg_hint);
}

cudaError_t dense_inverse(const float *in, long long in_pitch, float *out, long long out_pitch, int W, int H,
                          int J, int wavelet, float *scratch, cudaStream_t s, int *err, int seg_hint)
{
    return dense_inverse_levels(in, in_pitch, out, out_pitch, W, H, J, 1, wavelet, scratch, s, err, seg_hint);
}

// ------------------------------------------------- pipelined host frames

// A dense frame in host memory is copied in, transformed and copied out in
// row bands on three streams, so that the copies in and out (full duplex over
// the host link) overlap each other and the kernels.  The caller's frame is
// both input and output: a copy out to host rows waits until the copy in has
// read them.
//
// Forward: level-0 row bands run in order.  Each band reads its input rows
// (with the lifting warm-up) and, ahead of need, the host rows its LH and HH
// rows will overwrite, so the band's whole detail output can leave at once.
// Level 1 runs band by band behind level 0 as its LL1 rows appear, and its
// detail rows leave as soon as their host rows have been read; the levels
// below run on the small LL2 band and its quadrant is copied out last.
// Inverse: the top-left quadrant (LL1 and every coarser band) comes first,
// levels J..2 run, then level 1 runs band by band as its detail rows arrive
// and its output rows leave.
constexpr int kInvBands = 16;
constexpr long long kPipelineMinPixels = 1LL << 22;

static int host_bands()
{
    static const int n = [] {
        const char *e = getenv("DWT_GPU_HOST_BANDS");
        const int v = e ? atoi(e) : 0;
        return v >= 2 && v <= 256 ? v : 16;
    }();
    return n;
}

// Whether the GPU addresses pageable host memory itself through the host's
// page tables (address translation services, as on Grace-Blackwell).  Copies
// to and from pageable memory through the copy engines return only when
// done (device to host), which would stall the banded pipeline's host
// thread; a copy kernel stays asynchronous.  DWT_GPU_DIRECT_HOST=0 turns
// this off.
static bool pageable_direct()
{
    static const bool on = [] {
        int dev = 0, a = 0, b = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        const char *e = getenv("DWT_GPU_DIRECT_HOST");
        return a == 1 && b == 1 && !(e && e[0] == '0');
    }();
    return on;
}

// A copy of `rows` rows of `width` bytes between host and device memory: a
// copy kernel when the GPU addresses the host side directly (`kernel`), else
// the copy engines.
static cudaError_t copy_rows(bool kernel, void *dst, long long dpitch, const void *src, long long spitch,
                             long long width, long long rows, cudaMemcpyKind kind, cudaStream_t s)
{
    if (kernel) return launch_copy_rows(dst, dpitch, src, spitch, width, rows, s);
    return cudaMemcpy2DAsync(dst, size_t(dpitch), src, size_t(spitch), size_t(width), size_t(rows), kind, s);
}

// Host rows of the caller's frame: which copy in read each row, and the
// copies out waiting for their rows.  Copy and band events come from the
// lane's pool in order.
struct HostRows {
    Lane &c;
    cudaStream_t si, so;
    char *host;
    long long sx;
    float *dev;
    long long P;
    int W, H;
    bool direct;              // copies by kernel (host memory the GPU addresses itself)
    int n_ev = 0;
    std::vector<int> ev_of;   // lane event of the copy that read row r, -1 while unread
    struct Out {
        int r0, r1, c0, c1;  // host rows / columns
        const float *src;    // device address of (r0, c0), pitch P
        int ev;              // band event it follows
    };
    std::vector<Out> pending;

    HostRows(Lane &c_, char *host_, long long sx_, float *dev_, long long P_, int W_, int H_, bool direct_)
        : c(c_), si(c_.s_in), so(c_.s_out), host(host_), sx(sx_), dev(dev_), P(P_), W(W_), H(H_), direct(direct_),
          ev_of(H_, -1)
    {
    }

    cudaError_t record(cudaStream_t st, int &idx)
    {
        idx = n_ev++;
        cudaEvent_t e = c.event(idx);
        return e ? cudaEventRecord(e, st) : cudaErrorMemoryAllocation;
    }

    // Copies in every unread row of [r0, r1), one copy per run of unread rows.
    cudaError_t read(int r0, int r1)
    {
        r0 = std::max(r0, 0);
        r1 = std::min(r1, H);
        for (int r = r0; r < r1;) {
            if (ev_of[r] >= 0) {
                ++r;
                continue;
            }
            int e = r + 1;
            while (e < r1 && ev_of[e] < 0) ++e;
            cudaError_t err = copy_rows(direct, dev + r * P, P * 4, host + r * sx, sx, W * 4LL, e - r,
                                        cudaMemcpyHostToDevice, si);
            int idx = 0;
            if (err == cudaSuccess) err = record(si, idx);
            if (err != cudaSuccess) return err;
            for (int k = r; k < e; ++k) ev_of[k] = idx;
            r = e;
        }
        return cudaSuccess;
    }

    // Latest copy that read a row of [r0, r1); -2 if one of them is unread.
    int last_copy(int r0, int r1) const
    {
        r0 = std::max(r0, 0);
        r1 = std::min(r1, H);
        int last = -1;
        for (int r = r0; r < r1; ++r) {
            if (ev_of[r] < 0) return -2;
            last = std::max(last, ev_of[r]);
        }
        return last;
    }

    // Stream `st` waits until rows [r0, r1) are in.
    cudaError_t wait_rows(cudaStream_t st, int r0, int r1)
    {
        const int last = last_copy(r0, r1);
        if (last == -2) return cudaErrorInvalidValue;  // a scheduling bug: rows not read
        return last >= 0 ? cudaStreamWaitEvent(st, c.event(last), 0) : cudaSuccess;
    }

    void out(int r0, int r1, int c0, int c1, const float *src, int ev)
    {
        if (r1 > r0 && c1 > c0) pending.push_back({r0, r1, c0, c1, src, ev});
    }

    // Issues every pending copy out whose host rows have been read (all of
    // them when `all`: the caller has read every row by then).
    cudaError_t flush(bool all)
    {
        size_t keep = 0;
        for (size_t k = 0; k < pending.size(); ++k) {
            const Out &o = pending[k];
            const int last = last_copy(o.r0, o.r1);
            if (last == -2) {
                if (all) return cudaErrorInvalidValue;
                pending[keep++] = o;
                continue;
            }
            cudaError_t e = cudaStreamWaitEvent(so, c.event(o.ev), 0);
            if (e == cudaSuccess && last >= 0) e = cudaStreamWaitEvent(so, c.event(last), 0);
            if (e == cudaSuccess)
                e = copy_rows(direct, host + o.r0 * sx + o.c0 * 4LL, sx, o.src, P * 4, (o.c1 - o.c0) * 4LL,
                              o.r1 - o.r0, cudaMemcpyDeviceToHost, so);
            if (e != cudaSuccess) return e;
        }
        pending.resize(keep);
        return cudaSuccess;
    }
};

static int pipelined_forward(Lane &c, int wavelet, char *host, long long sx, int W, int H, int J, bool direct)
{
    cudaStream_t s = c.stream, si = c.s_in, so = c.s_out;
    const long long P = align_up(W, 32);
    Buf in(size_t(P) * H * 4 + 256, s), out(size_t(P) * H * 4 + 256, s);
    long long p0, p1;
    const size_t sf = dense_scratch_floats(W, H, J, &p0, &p1);
    Buf scratch(sf * 4 + 256, s);
    if (!in.p || !out.p || (sf && !scratch.p)) return set_error(DWT_GPU_ENOMEM);
    float *buf[2];
    long long p[2];
    scratch_frames(W, H, J, scratch.f(), buf, p);
    HostRows R(c, host, sx, in.f(), P, W, H, direct);
    // the pool may hand out blocks last used on `s`: let the copy streams wait
    int ev0 = 0;
    CK(R.record(s, ev0));
    CK(cudaStreamWaitEvent(si, c.event(ev0), 0));
    CK(cudaStreamWaitEvent(so, c.event(ev0), 0));

    const int LAT = wavelet == CDF97 ? 2 : 1;
    float *const o = out.f();
    // detail (and, at the last level, LL) output of level j's pairs [k0, k1)
    auto emit = [&](int j, int k0, int k1, int ev) {
        const int w = ceil_div_pow2(W, j), h = ceil_div_pow2(H, j);
        const int wd = (w + 1) / 2, hd = (h + 1) / 2, hh = h / 2;
        if (j == J - 1)
            R.out(k0, k1, 0, w, o + k0 * P, ev);  // LL and HL
        else
            R.out(k0, k1, wd, w, o + k0 * P + wd, ev);  // HL
        R.out(hd + k0, hd + std::min(k1, hh), 0, w, o + (hd + k0) * P, ev);  // LH, HH
    };

    LevelDesc d0 = fwd_desc(in.f(), P, o, P, W, H, J, 0, buf, p);
    plan_level(d0, 0, false);
    const int np0 = (H + 1) / 2, hd0 = np0, hh0 = H / 2, nb = host_bands();
    const int per0 = std::max(1, (d0.n_segs + nb - 1) / nb);
    const bool lvl1 = J >= 2;
    LevelDesc d1{};
    int np1 = 0, per1 = 1, next1 = 0;
    if (lvl1) {
        d1 = fwd_desc(in.f(), P, o, P, W, H, J, 1, buf, p);
        plan_level(d1, 0, false);
        np1 = (d1.h + 1) / 2;
        per1 = std::max(1, (d1.n_segs + nb / 2 - 1) / (nb / 2));
    }
    // level-1 segments whose LL1 rows (with the warm-up) are computed
    auto run_level1 = [&](int done0) -> cudaError_t {
        while (lvl1 && next1 < d1.n_segs) {
            const int se = std::min(d1.n_segs, next1 + per1);
            const int q0 = next1 * d1.seg_pairs, q1 = std::min(np1, se * d1.seg_pairs);
            if (done0 < d1.h && 2 * q1 + 2 * LAT > done0) break;
            LevelDesc d = d1;
            d.seg_base = next1;
            d.n_segs = se - next1;
            cudaError_t e = launch_level(d, wavelet, false, s, c.d_err);
            int ev = 0;
            if (e == cudaSuccess) e = R.record(s, ev);
            if (e != cudaSuccess) return e;
            emit(1, q0, q1, ev);
            next1 = se;
        }
        return cudaSuccess;
    };
    for (int sb = 0; sb < d0.n_segs; sb += per0) {
        const int se = std::min(d0.n_segs, sb + per0);
        const int k0 = sb * d0.seg_pairs, k1 = std::min(np0, se * d0.seg_pairs);
        // the band's input rows with the warm-up, then the host rows its LH
        // and HH rows overwrite
        CK(R.read(2 * k0 - 2 * LAT, 2 * k1 + 2 * LAT));
        CK(R.read(hd0 + k0, hd0 + std::min(k1, hh0)));
        CK(R.wait_rows(s, 2 * k0 - 2 * LAT, 2 * k1 + 2 * LAT));
        LevelDesc d = d0;
        d.seg_base = sb;
        d.n_segs = se - sb;
        CK(launch_level(d, wavelet, false, s, c.d_err));
        int ev = 0;
        CK(R.record(s, ev));
        emit(0, k0, k1, ev);
        CK(run_level1(k1));
        CK(R.flush(false));
    }
    CK(run_level1(np0));
    CK(R.flush(true));
    if (J > 2) {
        // levels 2 .. J-1 on LL2, then its quadrant (every coarser band)
        CK(dense_forward_levels(in.f(), P, o, P, W, H, J, 2, wavelet, scratch.f(), s, c.d_err, 0));
        int ev = 0;
        CK(R.record(s, ev));
        CK(cudaStreamWaitEvent(so, c.event(ev), 0));
        CK(copy_rows(direct, host, sx, o, P * 4, ceil_div_pow2(W, 2) * 4LL, ceil_div_pow2(H, 2),
                     cudaMemcpyDeviceToHost, so));
    }
    // buffers go back to the pool on `s`: order `s` after the copy-out
    int evo = 0;
    CK(R.record(so, evo));
    CK(cudaStreamWaitEvent(s, c.event(evo), 0));
    return set_error(lane_finish(c));
}

static int pipelined_inverse(Lane &c, int wavelet, char *host, long long sx, int W, int H, int J, bool direct)
{
    cudaStream_t s = c.stream, si = c.s_in, so = c.s_out;
    const long long P = align_up(W, 32);
    Buf in(size_t(P) * H * 4 + 256, s), out(size_t(P) * H * 4 + 256, s);
    long long p0, p1;
    const size_t sf = dense_scratch_floats(W, H, J, &p0, &p1);
    Buf scratch(sf * 4 + 256, s);
    if (!in.p || !out.p || (sf && !scratch.p)) return set_error(DWT_GPU_ENOMEM);
    float *buf[2];
    long long p[2];
    scratch_frames(W, H, J, scratch.f(), buf, p);
    int n_ev = 0;
    auto record = [&](cudaStream_t st) -> cudaEvent_t {
        cudaEvent_t e = c.event(n_ev++);
        return e && cudaEventRecord(e, st) == cudaSuccess ? e : nullptr;
    };
    cudaEvent_t e0 = record(s);
    if (!e0) return set_error(DWT_GPU_ECUDA);
    CK(cudaStreamWaitEvent(si, e0, 0));
    CK(cudaStreamWaitEvent(so, e0, 0));

    const int LAT = wavelet == CDF97 ? 2 : 1;
    const int ws = (W + 1) / 2, hs = (H + 1) / 2, hh = H / 2;
    // the top-left quadrant first: LL1 and every coarser band
    CK(copy_rows(direct, in.f(), P * 4, host, sx, ws * 4LL, hs, cudaMemcpyHostToDevice, si));
    cudaEvent_t eq = record(si);
    if (!eq) return set_error(DWT_GPU_ECUDA);
    CK(cudaStreamWaitEvent(s, eq, 0));
    if (J > 1) CK(dense_inverse_levels(in.f(), P, out.f(), P, W, H, J, 2, wavelet, scratch.f(), s, c.d_err, 0));

    LevelDesc d1 = inv_desc(in.f(), P, out.f(), P, W, H, J, 1, buf, p);
    plan_level(d1, 0, true);
    const int npairs = (H + 1) / 2, seg = d1.seg_pairs, nsegs = d1.n_segs;
    const int per_band = std::max(1, (nsegs + kInvBands - 1) / kInvBands);
    int top_in = 0, bot_in = 0;
    for (int sb = 0; sb < nsegs; sb += per_band) {
        const int se = std::min(nsegs, sb + per_band);
        const int k0 = sb * seg, k1 = std::min(npairs, se * seg);
        const int r0 = 2 * k0, r1 = std::min(H, 2 * k1);
        // the band rows the output pairs read (with the warm-up), and at least
        // every input row the band's output rows overwrite on the host
        int need_top = std::min(hs, k1 + LAT), need_bot = std::min(hh, k1 + LAT);
        need_top = std::max(need_top, std::min(hs, r1));
        need_bot = std::max(need_bot, std::min(hh, r1 - hs));
        if (need_top > top_in && W > ws)
            CK(copy_rows(direct, in.f() + top_in * P + ws, P * 4, host + top_in * sx + ws * 4LL, sx,
                         (W - ws) * 4LL, need_top - top_in, cudaMemcpyHostToDevice, si));
        if (need_bot > bot_in)
            CK(copy_rows(direct, in.f() + (hs + bot_in) * P, P * 4, host + (hs + bot_in) * sx, sx, W * 4LL,
                         need_bot - bot_in, cudaMemcpyHostToDevice, si));
        top_in = std::max(top_in, need_top);
        bot_in = std::max(bot_in, need_bot);
        cudaEvent_t ein = record(si);
        if (!ein) return set_error(DWT_GPU_ECUDA);
        CK(cudaStreamWaitEvent(s, ein, 0));
        LevelDesc d = d1;
        d.seg_base = sb;
        d.n_segs = se - sb;
        CK(launch_level(d, wavelet, true, s, c.d_err));
        cudaEvent_t eb = record(s);
        if (!eb) return set_error(DWT_GPU_ECUDA);
        // the output rows overwrite host rows whose input is already read
        CK(cudaStreamWaitEvent(so, eb, 0));
        CK(cudaStreamWaitEvent(so, ein, 0));
        CK(copy_rows(direct, host + r0 * sx, sx, out.f() + r0 * P, P * 4, W * 4LL, r1 - r0, cudaMemcpyDeviceToHost,
                     so));
    }
    cudaEvent_t eo = record(so);
    if (!eo) return set_error(DWT_GPU_ECUDA);
    CK(cudaStreamWaitEvent(s, eo, 0));
    return set_error(lane_finish(c));
}

// ------------------------------------------------ in place on device frames

// A dense device frame transformed in place (the reference's own calling
// convention, src/libdwt.h:491-502) without staging the whole frame.  Only
// level 0 -- the last level of the inverse -- has an in-place hazard: its
// tiles write the three detail quadrants (top right, bottom left, bottom
// right) where other tiles still read their input.  Every coarser level only
// reads the top-left quadrant and the LL scratch and writes the top-left
// quadrant, which level 0 no longer reads (forward) or does not touch until
// they are done (inverse).  So:
//   forward: level 0 reads the frame and writes the detail rows it may not
//            write in place yet to a staging frame T (LL1 to scratch); then,
//            on a second stream, those are copied from T into the frame while
//            levels 1 .. J-1 run on the first and write the top-left quadrant;
//   inverse: the detail rows level 0 could overwrite before reading them are
//            copied from the frame into T on a second stream while levels
//            J .. 2 read the top-left quadrant; level 0 then reads LL1, the
//            staged details from T and the others from the frame, and writes
//            the whole frame.
// Which rows need T follows from running level 0 in row bands in a fixed
// order (inplace_device): the HL quadrant and the LH / HH rows of the last
// one or two bands, about 3/8 of the frame read and written once (3 bytes per
// pixel) instead of 8 bytes per pixel for a staged copy of the whole frame,
// and the copies overlap the coarser, latency-bound levels.
constexpr long long kInPlaceMinPixels = 1LL << 20;

// DWT_GPU_SPARSE_FUSED=0 keeps sparse frames on the per-line sequence.
static bool sparse_enabled()
{
    static const bool on = [] {
        const char *v = getenv("DWT_GPU_SPARSE_FUSED");
        return !(v && v[0] == '0');
    }();
    return on;
}

// DWT_GPU_INPLACE=0 stages the whole frame instead (the general path).
static bool inplace_enabled()
{
    static const bool on = [] {
        const char *v = getenv("DWT_GPU_INPLACE");
        return !(v && v[0] == '0');
    }();
    return on;
}

static bool inplace_device_ok(const void *ptr, long long sx_bytes, int W, int H, int J)
{
    return J >= 2 && (long long)W * H >= kInPlaceMinPixels && (sx_bytes % 16) == 0 &&
           (reinterpret_cast<uintptr_t>(ptr) & 15) == 0 && coarse_level(W, H, J) >= 1;
}

// Level 0 of an in-place transform (the last level of the inverse) is one
// ordered launch: its units take tickets in segment order -- bottom-up in the
// forward, where a segment's LH / HH rows (hs + its pairs) lie below the rows
// it and every later segment reads; top-down in the inverse, where a segment
// reads LH / HH rows no earlier segment has written -- and each waits before
// it starts for the earlier segments that read the rows it overwrites
// (inplace_readers).  The segments at the end of the order, where that
// does not hold, are staged through T, and so is the HL quadrant, whose
// readers and writers run in the opposite order in both directions.  `lead`
// segments more are staged so that a unit seldom waits for one still running
// (DWT_GPU_INPLACE_LEAD, default kInPlaceLead).
constexpr int kInPlaceLead = 16;

static int inplace_lead()
{
    static const int n = [] {
        const char *e = getenv("DWT_GPU_INPLACE_LEAD");
        const int v = e ? atoi(e) : -1;
        return v >= 0 && v <= 4096 ? v : kInPlaceLead;
    }();
    return n;
}

// First staged segment of an ordered in-place level (segments >= it go
// through T): forward, the first segment (top-down) whose readers do not all
// come at least lead + 1 segments earlier in the bottom-up order; inverse,
// the largest bound that leaves every writer's in-frame readers at least
// lead + 1 segments earlier in the top-down order.
static int inplace_stage_seg(int h, int S, int nsegs, int lat, bool inverse, int lead, int dy)
{
    int a, b;
    if (!inverse) {
        for (int s = 0; s < nsegs; ++s) {
            inplace_readers(h, S, nsegs, lat, false, s, nsegs, dy, a, b);
            if (b >= a && a <= s + lead) return s;
        }
        return nsegs;
    }
    int st = nsegs;
    for (int w = 0; w < nsegs; ++w) {
        inplace_readers(h, S, nsegs, lat, true, w, nsegs, dy, a, b);
        if (b >= a && b > w - 1 - lead) st = std::min(st, w - lead);
    }
    return std::max(st, 0);
}

static int inplace_device(Lane &c, int wavelet, bool inverse, float *F, long long sx_bytes, int W, int H, int J)
{
    cudaStream_t s = c.stream, s2 = c.s_in;
    const long long Fp = sx_bytes / 4;
    const long long P = align_up(W, 32);
    const int ws = (W + 1) / 2, hs = (H + 1) / 2;
    const int LAT = wavelet == CDF97 ? 2 : 1;
    Buf T(size_t(P) * H * 4 + 256, s);
    long long p0, p1;
    const size_t sf = dense_scratch_floats(W, H, J, &p0, &p1);
    Buf scratch(sf * 4 + 256, s);
    if (!T.p || (sf && !scratch.p)) return set_error(DWT_GPU_ENOMEM);
    float *buf[2];
    long long p[2];
    scratch_frames(W, H, J, scratch.f(), buf, p);
    cudaEvent_t e_start = c.event(0), e_copy = c.event(1);
    if (!e_start || !e_copy) return set_error(DWT_GPU_ECUDA);

    // level 0 (forward) / the last inverse level: HL in T, LH / HH in the
    // frame except for the staged segments
    LevelDesc d0 = inverse ? inv_desc(T.f(), P, F, Fp, W, H, J, 1, buf, p)
                           : fwd_desc(F, Fp, T.f(), P, W, H, J, 0, buf, p);
    plan_level(d0, 0, inverse);
    const int S = d0.seg_pairs, nsegs = d0.n_segs;
    Buf order(size_t(nsegs + 1) * 4, s);
    if (!order.p) return set_error(DWT_GPU_ENOMEM);
    d0.order = static_cast<int *>(order.p);
    d0.seg_base = 0;
    d0.reverse = inverse ? 0 : 1;
    d0.order_dy = hs;
    d0.stage_seg = inplace_stage_seg(H, S, nsegs, LAT, inverse, inplace_lead(), hs);
    d0.alt[0] = T.f() + (long long)hs * P;
    d0.alt[1] = T.f() + (long long)hs * P + ws;
    d0.alt_pitch = P;
    float *const lh = F + (long long)hs * Fp, *const hh = F + (long long)hs * Fp + ws;
    if (!inverse) {
        d0.out[2] = lh;
        d0.out[3] = hh;
        d0.out_pitch[2] = d0.out_pitch[3] = Fp;
    } else {
        d0.in[2] = lh;
        d0.in[3] = hh;
        d0.in_pitch[2] = d0.in_pitch[3] = Fp;
    }
    // LH / HH rows that pass through T: [staged_lo, H)
    long long staged_lo = H;
    if (d0.stage_seg < nsegs) {
        const long long k = (long long)d0.stage_seg * S;
        staged_lo = inverse ? hs + std::max(0LL, k - LAT - 3) : hs + k;
        staged_lo = std::min<long long>(H, std::max<long long>(hs, staged_lo));
    }
    // the HL quadrant and the staged LH / HH rows between the frame and T
    auto copy_staged = [&](float *dst, long long dp, const float *src, long long sp) -> cudaError_t {
        cudaError_t e = cudaSuccess;
        if (W > ws) e = launch_copy_rows_bulk(dst + ws, dp * 4, src + ws, sp * 4, (W - ws) * 4LL, hs, s2, c.d_err);
        if (e == cudaSuccess && staged_lo < H)
            e = launch_copy_rows_bulk(dst + staged_lo * dp, dp * 4, src + staged_lo * sp, sp * 4, W * 4LL,
                                      H - staged_lo, s2, c.d_err);
        return e;
    };
    CK(cudaMemsetAsync(order.p, 0, size_t(nsegs + 1) * 4, s));
    if (!inverse) {
        // the copy back starts after level 1 (HBM-bound like the copy) and
        // runs beside the latency-bound smaller levels
        CK(launch_level(d0, wavelet, false, s, c.d_err));
        const bool levels = coarse_level(W, H, J) > 1;
        if (!levels) CK(cudaEventRecord(e_start, s));
        CK(dense_forward_levels(F, Fp, F, Fp, W, H, J, 1, wavelet, scratch.f(), s, c.d_err, 0,
                                levels ? e_start : nullptr));
        CK(cudaStreamWaitEvent(s2, e_start, 0));
        CK(copy_staged(F, Fp, T.f(), P));
        CK(cudaEventRecord(e_copy, s2));
        CK(cudaStreamWaitEvent(s, e_copy, 0));
    } else {
        CK(cudaEventRecord(e_start, s));
        CK(cudaStreamWaitEvent(s2, e_start, 0));
        CK(copy_staged(T.f(), P, F, Fp));
        CK(cudaEventRecord(e_copy, s2));
        CK(dense_inverse_levels(F, Fp, F, Fp, W, H, J, 2, wavelet, scratch.f(), s, c.d_err, 0));
        CK(cudaStreamWaitEvent(s, e_copy, 0));
        CK(launch_level(d0, wavelet, true, s, c.d_err));
    }
    return set_error(lane_finish(c));
}

// ----------------------------------------- sparse frames with zero padding

// An outer ox x oy frame holding an ix x iy inner image (the SIMPLE / SPARSE
// layouts of src/libdwt.c:8620-8659, and the OpenCV wrapper's padding,
// src/cvdwt.cpp:149-181), transformed in place with zero padding.  Per level
// the reference transforms every row of the outer frame over the inner
// length, then every column, writing H at the OUTER midpoint, and zeroes the
// rest of the level's frame (src/libdwt.c:6353-6397, 6700-6745).  Everything
// it computes outside the inner bands is then overwritten or zeroed, so the
// result is the dense level of the inner frame with its H bands at the outer
// midpoints, and zeros everywhere no band of any level lands.  The fused
// level kernel does the large levels that way (level 0 -- the last inverse
// level -- through the staging frame T, as for dense frames in place); the
// small ones run the reference's per-line sequence in place, and a last kernel
// writes the zeros.
static bool sparse_fast_level(int iw, int ih) { return iw >= 16 && ih >= 16 && (long long)iw * ih > 4096; }

static bool sparse_fast_ok(const void *F, long long Fp, int ox, int oy, int ix, int iy, int J)
{
    return J >= 1 && sparse_fast_level(ix, iy) && (Fp % 4) == 0 && (reinterpret_cast<uintptr_t>(F) & 15) == 0 &&
           ox >= ix && oy >= iy;
}

// Rectangles [x0, x1) x [y0, y1) of zero fill.
struct ZRect {
    int x0, y0, x1, y1;
    bool empty() const { return x1 <= x0 || y1 <= y0; }
};

static ZRect zrect_and(const ZRect &a, const ZRect &b)
{
    return ZRect{std::max(a.x0, b.x0), std::max(a.y0, b.y0), std::min(a.x1, b.x1), std::min(a.y1, b.y1)};
}

// The parts of every rectangle of `in` outside k (up to four pieces each).
static std::vector<ZRect> zrect_minus(const std::vector<ZRect> &in, const ZRect &k)
{
    std::vector<ZRect> out;
    for (const ZRect &a : in) {
        const ZRect c = zrect_and(a, k);
        if (a.empty()) continue;
        if (c.empty()) {
            out.push_back(a);
            continue;
        }
        const ZRect pieces[4] = {{a.x0, a.y0, a.x1, c.y0},     // above
                                 {a.x0, c.y1, a.x1, a.y1},     // below
                                 {a.x0, c.y0, c.x0, c.y1},     // left
                                 {c.x1, c.y0, a.x1, c.y1}};    // right
        for (const ZRect &p : pieces)
            if (!p.empty()) out.push_back(p);
    }
    return out;
}

static void zrects_add(ZeroRects &Z, const ZRect &r)
{
    if (r.empty() || Z.n >= kMaxZeroRects) return;
    Z.x0[Z.n] = r.x0;
    Z.y0[Z.n] = r.y0;
    Z.w[Z.n] = r.x1 - r.x0;
    Z.first_row[Z.n] = Z.total_rows;
    Z.total_rows += r.y1 - r.y0;
    Z.n++;
}

static int sparse_inplace(Lane &c, int wavelet, bool inverse, float *F, long long Fp, int ox, int oy, int ix,
                          int iy, int J)
{
    cudaStream_t s = c.stream, s2 = c.s_in;
    auto cdp = [](int v, int j) { return ceil_div_pow2(v, j); };
    const long long P = align_up(ox, 32);
    Buf T(size_t(P) * oy * 4 + 256, s);
    // LL ping-pong frames as the dense pipeline lays them out; with one level
    // the forward still stages LL1 in the first of them
    const int Js = std::max(J, 2);
    long long p0, p1;
    const size_t sf = dense_scratch_floats(ix, iy, Js, &p0, &p1);
    Buf scratch(sf * 4 + 256, s);
    if (!T.p || !scratch.p) return set_error(DWT_GPU_ENOMEM);
    float *buf[2];
    long long p[2];
    scratch_frames(ix, iy, Js, scratch.f(), buf, p);
    cudaEvent_t e_start = c.event(0), e_copy = c.event(1);
    if (!e_start || !e_copy) return set_error(DWT_GPU_ECUDA);
    // Level 0 (the last inverse level) is an ordered in-place launch as for
    // dense frames, with the LH / HH bands at the outer midpoint row ody:
    // HL and the LH / HH rows of the staged segments pass through T (same
    // positions).
    const int odx = cdp(ox, 1), ody = cdp(oy, 1);
    const int lx = (ix + 1) / 2, hx = ix / 2, ly = (iy + 1) / 2, hy = iy / 2;
    const int LAT = wavelet == CDF97 ? 2 : 1;
    Buf order;
    ZeroRects late_zeros{};
    long long staged_lo = (long long)ody + hy;  // LH / HH rows [staged_lo, ody + hy) pass through T
    auto order_level0 = [&](LevelDesc &d, bool inv, int dx, int dy, float *Tb, long long tp, float *Fb,
                            long long fp) -> cudaError_t {
        const int S = d.seg_pairs, nsegs = d.n_segs;
        if (!order.p && !order.alloc(size_t(nsegs + 1) * 4, s)) return cudaErrorMemoryAllocation;
        d.order = static_cast<int *>(order.p);
        d.seg_base = 0;
        d.reverse = inv ? 0 : 1;
        d.order_dy = dy;
        d.stage_seg = inplace_stage_seg(d.h, S, nsegs, LAT, inv, inplace_lead(), dy);
        d.alt[0] = Tb + (long long)dy * tp;
        d.alt[1] = Tb + (long long)dy * tp + dx;
        d.alt_pitch = tp;
        float *lh = Fb + (long long)dy * fp, *hh = Fb + (long long)dy * fp + dx;
        if (!inv) {
            d.out[2] = lh;
            d.out[3] = hh;
            d.out_pitch[2] = d.out_pitch[3] = fp;
        } else {
            d.in[2] = lh;
            d.in[3] = hh;
            d.in_pitch[2] = d.in_pitch[3] = fp;
        }
        if (d.stage_seg < nsegs) {
            const long long k = (long long)d.stage_seg * S;
            staged_lo = inv ? dy + std::max(0LL, k - LAT - 3) : dy + k;
            staged_lo = std::min<long long>((long long)dy + hy, std::max<long long>(dy, staged_lo));
        } else {
            staged_lo = (long long)dy + hy;
        }
        return cudaMemsetAsync(order.p, 0, size_t(nsegs + 1) * 4, s);
    };
    auto copy_details = [&](float *dst, long long dp, const float *src, long long sp) -> cudaError_t {
        cudaError_t e = cudaSuccess;
        auto rect = [&](int x0, long long y0, int w, long long h) {
            if (e == cudaSuccess && w > 0 && h > 0)
                e = launch_copy_rows_bulk(dst + y0 * dp + x0, dp * 4, src + y0 * sp + x0, sp * 4, w * 4LL, h, s2,
                                          c.d_err);
        };
        const long long rows = (long long)ody + hy - staged_lo;
        rect(odx, 0, hx, ly);             // HL
        rect(0, staged_lo, lx, rows);     // LH of the staged segments
        rect(odx, staged_lo, hx, rows);   // HH of the staged segments
        return e;
    };
    // tmp of the per-line levels: lines x length of the largest such frame
    auto line_tmp = [&](int j) { return size_t(std::max(cdp(ox, j), cdp(oy, j))) * std::max(cdp(ox, j), cdp(oy, j)); };
    if (!inverse) {
        int jf = 0;  // levels 0 .. jf-1 fused, the rest per line
        while (jf < J && sparse_fast_level(cdp(ix, jf), cdp(iy, jf))) ++jf;
        Buf tmp(jf < J ? line_tmp(jf) * 4 + 256 : 256, s);
        if (!tmp.p) return set_error(DWT_GPU_ENOMEM);
        for (int j = 0; j < jf; ++j) {
            LevelDesc d{};
            d.w = cdp(ix, j);
            d.h = cdp(iy, j);
            d.in[0] = j == 0 ? F : buf[(j - 1) % 2];
            d.in_pitch[0] = j == 0 ? Fp : p[(j - 1) % 2];
            const bool ll_to_frame = j == jf - 1 && j >= 1;
            d.out[0] = ll_to_frame ? F : buf[j % 2];
            d.out_pitch[0] = ll_to_frame ? Fp : p[j % 2];
            float *base = j == 0 ? T.f() : F;
            const long long bp = j == 0 ? P : Fp;
            const int dx = cdp(ox, j + 1), dy = cdp(oy, j + 1);
            d.out[1] = base + dx;
            d.out[2] = base + dy * bp;
            d.out[3] = base + dy * bp + dx;
            d.out_pitch[1] = d.out_pitch[2] = d.out_pitch[3] = bp;
            plan_level(d, 0, false);
            d.reverse = kAlternateOrder && (j & 1);
            if (j == 0) {
                // ordered level 0: LH / HH into the frame but for the staged segments
                CK(order_level0(d, false, dx, dy, T.f(), P, F, Fp));
            }
            CK(launch_level(d, wavelet, false, s, c.d_err));
            if (j == 0) {
                CK(cudaEventRecord(e_start, s));
                CK(cudaStreamWaitEvent(s2, e_start, 0));
                CK(copy_details(F, Fp, T.f(), P));
                if (jf == 1)  // LL1 into the frame for the per-line levels
                    CK(launch_copy_rows_dev(F, Fp * 4, buf[0], p[0] * 4, lx * 4LL, ly, s));
            }
        }
        if (jf < J && sparse_tail_smem(ox, oy, jf) <= kSparseTailSmem) {
            CK(launch_sparse_tail(false, F, Fp, ox, oy, ix, iy, jf, J, wavelet, s));
        } else {
            for (int j = jf; j < J; ++j)
                CK(sparse_forward_level(F, Fp, cdp(ox, j), cdp(oy, j), cdp(ox, j + 1), cdp(oy, j + 1), cdp(ix, j),
                                        cdp(iy, j), 1, wavelet, tmp.f(), s));
        }
        // zeros where no band of the fused levels lands (the per-line levels
        // zero their own frames): per fused level, the parts of its frame
        // outside its four bands and outside the next level's frame.  Level
        // 0's parts lie outside the frame of every later level: they are
        // written on the second stream after level 0, beside the smaller levels
        ZeroRects R0{}, R{};
        auto add = [&](ZeroRects &Z, int x0, int y0, int w, int h) {
            if (w <= 0 || h <= 0 || Z.n >= kMaxZeroRects) return;
            Z.x0[Z.n] = x0;
            Z.y0[Z.n] = y0;
            Z.w[Z.n] = w;
            Z.first_row[Z.n] = Z.total_rows;
            Z.total_rows += h;
            Z.n++;
        };
        for (int j = 0; j < jf; ++j) {
            ZeroRects &Z = j == 0 ? R0 : R;
            const int ow = cdp(ox, j), oh = cdp(oy, j), dx = cdp(ox, j + 1), dy = cdp(oy, j + 1);
            const int iw = cdp(ix, j), ih = cdp(iy, j);
            const int lxj = (iw + 1) / 2, hxj = iw / 2, lyj = (ih + 1) / 2, hyj = ih / 2;
            add(Z, lxj, dy, dx - lxj, oh - dy);         // between the L and H columns, below the next frame
            add(Z, dx + hxj, 0, ow - dx - hxj, oh);     // right of the H columns
            add(Z, dx, lyj, hxj, dy - lyj);             // H columns, between the L and H rows
            add(Z, 0, dy + hyj, lxj, oh - dy - hyj);    // L columns, below the H rows
            add(Z, dx, dy + hyj, hxj, oh - dy - hyj);   // H columns, below the H rows
            if (j == J - 1) {                           // the last level's frame around LL_J
                add(R, lxj, 0, dx - lxj, dy);
                add(R, 0, lyj, lxj, dy - lyj);
            }
        }
        CK(launch_zero_rects(F, Fp, R0, s2));
        CK(cudaEventRecord(e_copy, s2));
        CK(cudaStreamWaitEvent(s, e_copy, 0));
        CK(launch_zero_rects(F, Fp, R, s));
    } else {
        // inverse level j rebuilds LL_{j-1} (cdp(i, j-1)) from LL_j and the
        // level's details at the outer midpoints cdp(o, j); levels 1 .. jf
        // fused, J .. jf+1 per line (first)
        int jf = 0;
        while (jf < J && sparse_fast_level(cdp(ix, jf), cdp(iy, jf))) ++jf;
        Buf tmp(jf < J ? line_tmp(jf) * 4 + 256 : 256, s);
        if (!tmp.p) return set_error(DWT_GPU_ENOMEM);
        {
            // the last level, planned first: the staged rows it reads from T
            LevelDesc d{};
            d.w = ix;
            d.h = iy;
            plan_level(d, 0, true);
            CK(order_level0(d, true, odx, ody, T.f(), P, F, Fp));
        }
        ZeroRects early_zeros{};
        {
            const ZRect outside[2] = {{ix, 0, ox, oy}, {0, iy, ix, oy}};
            const ZRect kept[4] = {{0, 0, odx, ody},                     // the coarser levels' quadrant
                                   {odx, 0, odx + hx, ly},               // HL of level 0
                                   {0, ody, lx, ody + hy},               // LH
                                   {odx, ody, odx + hx, ody + hy}};      // HH
            std::vector<ZRect> early(outside, outside + 2);
            for (const ZRect &k : kept) early = zrect_minus(early, k);
            if (early.size() <= size_t(kMaxZeroRects) / 2) {
                for (const ZRect &e : early) zrects_add(early_zeros, e);
                for (const ZRect &o : outside)
                    for (const ZRect &k : kept) zrects_add(late_zeros, zrect_and(o, k));
            } else {  // (not met by the band layout) everything after level 0
                for (const ZRect &o : outside) zrects_add(late_zeros, o);
            }
        }
        CK(cudaEventRecord(e_start, s));
        CK(cudaStreamWaitEvent(s2, e_start, 0));
        CK(copy_details(T.f(), P, F, Fp));
        CK(launch_zero_rects(F, Fp, early_zeros, s2));
        CK(cudaEventRecord(e_copy, s2));
        if (jf < J && sparse_tail_smem(ox, oy, jf) <= kSparseTailSmem) {
            CK(launch_sparse_tail(true, F, Fp, ox, oy, ix, iy, jf, J, wavelet, s));
        } else {
            for (int j = J; j > jf; --j)
                CK(sparse_inverse_level(F, Fp, cdp(ox, j), cdp(oy, j), cdp(ox, j - 1), cdp(oy, j - 1),
                                        cdp(ix, j - 1), cdp(iy, j - 1), 1, wavelet, tmp.f(), s));
        }
        for (int j = jf; j >= 1; --j) {
            LevelDesc d{};
            d.w = cdp(ix, j - 1);
            d.h = cdp(iy, j - 1);
            d.in[0] = j == jf ? F : buf[(j - 1) % 2];
            d.in_pitch[0] = j == jf ? Fp : p[(j - 1) % 2];
            if (j == 1 && jf == 1) {
                // level 0 writes the frame rows LL_1 sits in: read LL_1 from scratch
                CK(launch_copy_rows_dev(buf[0], p[0] * 4, F, Fp * 4, cdp(ix, 1) * 4LL, cdp(iy, 1), s));
                d.in[0] = buf[0];
                d.in_pitch[0] = p[0];
            }
            const float *base = j == 1 ? T.f() : F;
            const long long bp = j == 1 ? P : Fp;
            const int sx = cdp(ox, j), sy = cdp(oy, j);
            d.in[1] = base + sx;
            d.in[2] = base + sy * bp;
            d.in[3] = base + sy * bp + sx;
            d.in_pitch[1] = d.in_pitch[2] = d.in_pitch[3] = bp;
            d.out[0] = j == 1 ? F : buf[(j - 2) % 2];
            d.out_pitch[0] = j == 1 ? Fp : p[(j - 2) % 2];
            plan_level(d, 0, true);
            d.reverse = kAlternateOrder && ((jf - j) & 1);
            if (j == 1) {
                CK(order_level0(d, true, sx, sy, T.f(), P, F, Fp));
                CK(cudaStreamWaitEvent(s, e_copy, 0));
            }
            CK(launch_level(d, wavelet, true, s, c.d_err));
        }
        // zero padding of the last level, everything outside the inner image:
        // the parts inside the level-0 detail bands or the top-left quadrant
        // (read by the inverse levels) after level 0, the rest -- read by
        // nothing -- written on the second stream up front (below)
        CK(launch_zero_rects(F, Fp, late_zeros, s));
    }
    return DWT_GPU_OK;
}

// ------------------------------------------------------------ 2D driver

// Validates a caller frame; returns false (and logs) for layouts the
// library does not take: non-positive sizes with levels to do, negative
// strides, samples that overlap, an inner frame larger than the outer one.
static bool frame_ok(int sx, int sy, int ox, int oy, int ix, int iy, int elem = 4)
{
    if (ox < 0 || oy < 0 || ix < 0 || iy < 0) {
        log_error("negative image size\n");
        return false;
    }
    if (ix > ox || iy > oy) {
        log_error("inner image %dx%d larger than the outer frame %dx%d\n", ix, iy, ox, oy);
        return false;
    }
    if (sx <= 0 || sy <= 0) {
        log_error("strides must be positive (stride_x=%d, stride_y=%d)\n", sx, sy);
        return false;
    }
    const bool rows = (long long)sy >= elem && (long long)sx >= (long long)ox * sy;
    const bool cols = (long long)sx >= elem && (long long)sy >= (long long)oy * sx;
    if (!(rows || cols) && ox > 1 && oy > 1) {
        log_error("stride_x=%d / stride_y=%d make samples of a %dx%d frame overlap\n", sx, sy, ox, oy);
        return false;
    }
    return true;
}

static long long span_bytes(int sx, int sy, int ox, int oy)
{
    return (long long)(oy - 1) * sx + (long long)(ox - 1) * sy + 4;
}

// The whole 2D call.  inverse: j is the requested level count (in); forward:
// *jp is clamped and written back first.
static int run_2d(int wavelet, bool inverse, void *ptr, int sx, int sy, int ox, int oy, int ix, int iy,
                  int *jp, int j_in, int decompose_one, int zero_padding)
{
    t_last_error = DWT_GPU_OK;
    if (!frame_ok(sx, sy, ox, oy, ix, iy)) return set_error(DWT_GPU_EINVAL);
    const int omin = std::min(ox, oy), omax = std::max(ox, oy);
    const int j_limit = (decompose_one ? omax : omin) > 0 ? ceil_log2_int(decompose_one ? omax : omin) : 0;
    int J;
    if (!inverse) {
        if (*jp < 0 || *jp > j_limit) *jp = j_limit;
        J = *jp;
    } else {
        J = j_limit;
        if (j_in >= 0 && j_in < J) J = j_in;
    }
    if (J == 0 || ox == 0 || oy == 0) return DWT_GPU_OK;
    if (!ptr) {
        log_error("null image pointer\n");
        return set_error(DWT_GPU_EINVAL);
    }

    const NvtxRange range("dwt 2D %s %s %dx%d j=%d", wavelet == CDF97 ? "cdf97" : "cdf53",
                          inverse ? "inverse" : "forward", ix, iy, J);
    LaneGuard lane_guard(ctx());
    Lane &c = lane_guard.get();
    cudaStream_t s = c.stream;
    const MemKind kind = classify(ptr);
    const bool on_device = kind == MemKind::Device || kind == MemKind::Managed;
    // pageable host memory the kernels address themselves
    const bool host_direct = kind == MemKind::Pageable && pageable_direct();
    const bool dense = (ix == ox && iy == oy);
    const long long P = align_up(ox, 32);  // compact pitch in floats
    // a single-row frame may carry any row stride; 2D copies want pitch >= width
    const long long csx = oy == 1 ? std::max<long long>(sx, 4LL * ox) : sx;

    // large dense host frames: banded copy/compute overlap
    {
        const bool rows4h = sy == 4 && (csx % 4) == 0 && (reinterpret_cast<uintptr_t>(ptr) & 3) == 0;
        if (!on_device && dense && rows4h && (long long)ox * oy >= kPipelineMinPixels && oy >= 64) {
            return inverse ? pipelined_inverse(c, wavelet, static_cast<char *>(ptr), csx, ox, oy, J, host_direct)
                           : pipelined_forward(c, wavelet, static_cast<char *>(ptr), csx, ox, oy, J, host_direct);
        }
    }

    // dense, aligned device frames: in place, staging only level 0's details
    if (on_device && dense && sy == 4 && inplace_device_ok(ptr, csx, ox, oy, J) && inplace_enabled())
        return inplace_device(c, wavelet, inverse, static_cast<float *>(ptr), csx, ox, oy, J);
    // sparse, zero-padded, aligned device frames: in place likewise
    const bool sparse_fast = !dense && zero_padding && sparse_enabled();
    if (on_device && sparse_fast && sy == 4 && (csx % 16) == 0 &&
        sparse_fast_ok(ptr, csx / 4, ox, oy, ix, iy, J)) {
        const int rc = sparse_inplace(c, wavelet, inverse, static_cast<float *>(ptr), csx / 4, ox, oy, ix, iy, J);
        if (rc != DWT_GPU_OK) return rc;
        return set_error(lane_finish(c));
    }

    // 1. stage into IN
    Buf in(size_t(P) * oy * 4 + 256, s);
    if (!in.p) return set_error(DWT_GPU_ENOMEM);
    Buf span;  // host path with a non-4-byte pixel pitch: device copy of the byte span
    const long long sb = span_bytes(sx, sy, ox, oy);
    // 2D copies take rows of whole, 4-byte aligned floats; anything else goes
    // through a byte span and the repack kernel
    const bool rows4 = sy == 4 && (csx % 4) == 0 && (reinterpret_cast<uintptr_t>(ptr) & 3) == 0;
    if (host_direct) {
        if (rows4)
            CK(launch_copy_rows(in.p, P * 4, ptr, csx, ox * 4LL, oy, s));
        else
            CK(launch_repack(ptr, sx, sy, ox, oy, in.f(), P, s));
    } else if (!on_device) {
        if (rows4) {
            CK(cudaMemcpy2DAsync(in.p, P * 4, ptr, csx, size_t(ox) * 4, oy, cudaMemcpyHostToDevice, s));
        } else {
            if (!span.alloc(size_t(sb) + 16, s)) return set_error(DWT_GPU_ENOMEM);
            CK(cudaMemcpyAsync(span.p, ptr, size_t(sb), cudaMemcpyHostToDevice, s));
            CK(launch_repack(span.p, sx, sy, ox, oy, in.f(), P, s));
        }
    } else if (rows4) {
        CK(cudaMemcpy2DAsync(in.p, P * 4, ptr, csx, size_t(ox) * 4, oy, cudaMemcpyDeviceToDevice, s));
    } else {
        CK(launch_repack(ptr, sx, sy, ox, oy, in.f(), P, s));
    }

    // 2. transform
    float *out = nullptr;
    long long out_pitch = 0;
    Buf outb;
    const bool direct = on_device && dense && rows4;
    if (dense) {
        if (direct) {
            out = static_cast<float *>(ptr);
            out_pitch = csx / 4;
        } else {
            if (!outb.alloc(size_t(P) * oy * 4 + 256, s)) return set_error(DWT_GPU_ENOMEM);
            out = outb.f();
            out_pitch = P;
        }
        long long p0, p1;
        const size_t sf = dense_scratch_floats(ox, oy, J, &p0, &p1);
        Buf scratch(sf * 4 + 256, s);
        if (sf && !scratch.p) return set_error(DWT_GPU_ENOMEM);
        if (!inverse)
            CK(dense_forward(in.f(), P, out, out_pitch, ox, oy, J, wavelet, scratch.f(), s, c.d_err, 0));
        else
            CK(dense_inverse(in.f(), P, out, out_pitch, ox, oy, J, wavelet, scratch.f(), s, c.d_err, 0));
    } else if (sparse_fast && sparse_fast_ok(in.f(), P, ox, oy, ix, iy, J)) {
        // sparse frame with zero padding: fused levels, in place on IN
        const int rc = sparse_inplace(c, wavelet, inverse, in.f(), P, ox, oy, ix, iy, J);
        if (rc != DWT_GPU_OK) return rc;
        out = in.f();
        out_pitch = P;
    } else {
        // sparse frame: the reference's per-line sequence, in place on IN
        const int lmax = std::max(ox, oy);
        Buf tmp(size_t(lmax) * lmax * 4 + 256, s);
        if (!tmp.p) return set_error(DWT_GPU_ENOMEM);
        if (!inverse) {
            for (int j = 0; j < J; ++j) {
                CK(sparse_forward_level(in.f(), P, ceil_div_pow2(ox, j), ceil_div_pow2(oy, j),
                                        ceil_div_pow2(ox, j + 1), ceil_div_pow2(oy, j + 1),
                                        ceil_div_pow2(ix, j), ceil_div_pow2(iy, j), zero_padding,
                                        wavelet, tmp.f(), s));
            }
        } else {
            for (int j = J; j >= 1; --j) {
                CK(sparse_inverse_level(in.f(), P, ceil_div_pow2(ox, j), ceil_div_pow2(oy, j),
                                        ceil_div_pow2(ox, j - 1), ceil_div_pow2(oy, j - 1),
                                        ceil_div_pow2(ix, j - 1), ceil_div_pow2(iy, j - 1), zero_padding,
                                        wavelet, tmp.f(), s));
            }
        }
        out = in.f();
        out_pitch = P;
    }

    // 3. write back
    if (host_direct) {
        if (rows4)
            CK(launch_copy_rows(ptr, csx, out, out_pitch * 4, ox * 4LL, oy, s));
        else
            CK(launch_unpack(out, out_pitch, ptr, sx, sy, ox, oy, s));
    } else if (!on_device) {
        if (rows4) {
            CK(cudaMemcpy2DAsync(ptr, csx, out, out_pitch * 4, size_t(ox) * 4, oy, cudaMemcpyDeviceToHost, s));
        } else {
            CK(launch_unpack(out, out_pitch, span.p, sx, sy, ox, oy, s));
            CK(cudaMemcpyAsync(ptr, span.p, size_t(sb), cudaMemcpyDeviceToHost, s));
        }
    } else if (!direct) {
        CK(launch_unpack(out, out_pitch, ptr, sx, sy, ox, oy, s));
    }
    return set_error(lane_finish(c));
}

// ------------------------------------------------------------ 1D driver

// The double-precision 2D call (libdwt's _2f_d / _2i_d): the frame's byte
// span staged to the device, repacked to a compact double frame, the
// reference's per-line level sequence in place (dense frames included), and
// unpacked back.  Same level and frame semantics as run_2d.
static int run_2d_d(int wavelet, bool inverse, void *ptr, int sx, int sy, int ox, int oy, int ix, int iy, int *jp,
                    int j_in, int decompose_one, int zero_padding)
{
    t_last_error = DWT_GPU_OK;
    if (!frame_ok(sx, sy, ox, oy, ix, iy, 8)) return set_error(DWT_GPU_EINVAL);
    const int omin = std::min(ox, oy), omax = std::max(ox, oy);
    const int j_limit = (decompose_one ? omax : omin) > 0 ? ceil_log2_int(decompose_one ? omax : omin) : 0;
    int J;
    if (!inverse) {
        if (*jp < 0 || *jp > j_limit) *jp = j_limit;
        J = *jp;
    } else {
        J = j_limit;
        if (j_in >= 0 && j_in < J) J = j_in;
    }
    if (J == 0 || ox == 0 || oy == 0) return DWT_GPU_OK;
    if (!ptr) {
        log_error("null image pointer\n");
        return set_error(DWT_GPU_EINVAL);
    }
    LaneGuard lane_guard(ctx());
    Lane &c = lane_guard.get();
    cudaStream_t s = c.stream;
    const MemKind kind = classify(ptr);
    const bool on_device = kind == MemKind::Device || kind == MemKind::Managed;
    const long long P = align_up(ox, 16);  // compact pitch in doubles
    const long long sb = (long long)(oy - 1) * sx + (long long)(ox - 1) * sy + 8;
    Buf frame(size_t(P) * oy * 8 + 256, s), span;
    if (!frame.p) return set_error(DWT_GPU_ENOMEM);
    double *f = static_cast<double *>(frame.p);
    const void *src = ptr;
    if (!on_device) {
        if (!span.alloc(size_t(sb) + 16, s)) return set_error(DWT_GPU_ENOMEM);
        CK(cudaMemcpyAsync(span.p, ptr, size_t(sb), cudaMemcpyHostToDevice, s));
        src = span.p;
    }
    CK(launch_repack_d(src, sx, sy, ox, oy, f, P, s));
    const int lmax = std::max(ox, oy);
    Buf tmp(size_t(lmax) * lmax * 8 + 256, s);
    if (!tmp.p) return set_error(DWT_GPU_ENOMEM);
    double *t = static_cast<double *>(tmp.p);
    if (!inverse) {
        for (int j = 0; j < J; ++j)
            CK(level_forward_d(f, P, ceil_div_pow2(ox, j), ceil_div_pow2(oy, j), ceil_div_pow2(ox, j + 1),
                               ceil_div_pow2(oy, j + 1), ceil_div_pow2(ix, j), ceil_div_pow2(iy, j), zero_padding,
                               wavelet, t, s));
    } else {
        for (int j = J; j >= 1; --j)
            CK(level_inverse_d(f, P, ceil_div_pow2(ox, j), ceil_div_pow2(oy, j), ceil_div_pow2(ox, j - 1),
                               ceil_div_pow2(oy, j - 1), ceil_div_pow2(ix, j - 1), ceil_div_pow2(iy, j - 1),
                               zero_padding, wavelet, t, s));
    }
    if (!on_device) {
        CK(launch_unpack_d(f, P, span.p, sx, sy, ox, oy, s));
        CK(cudaMemcpyAsync(ptr, span.p, size_t(sb), cudaMemcpyDeviceToHost, s));
    } else {
        CK(launch_unpack_d(f, P, ptr, sx, sy, ox, oy, s));
    }
    return set_error(lane_finish(c));
}

// The double-precision strided 1D level (libdwt's _ex_stride_d): the samples
// gathered into one compact line, transformed, scattered to dst_l / dst_h
// (forward) or dst (inverse).
static int run_1d_d(int wavelet, bool inverse, const double *a, const double *b, double *c_l, double *h_out,
                    int N, int stride)
{
    t_last_error = DWT_GPU_OK;
    if (N < 0 || stride == 0) {
        log_error("invalid 1D arguments (N=%d, stride=%d)\n", N, stride);
        return set_error(DWT_GPU_EINVAL);
    }
    if (N == 0) return DWT_GPU_OK;
    if (stride < 8) {
        log_error("stride %d smaller than a sample\n", stride);
        return set_error(DWT_GPU_EINVAL);
    }
    LaneGuard lane_guard(ctx());
    Lane &c = lane_guard.get();
    cudaStream_t s = c.stream;
    const int nl = (N + 1) / 2, nh = N / 2;
    Buf line(size_t(N) * 8 + 256, s), tmp(size_t(N) * 8 + 256, s);
    if (!line.p || !tmp.p) return set_error(DWT_GPU_ENOMEM);
    double *x = static_cast<double *>(line.p);
    // samples at `stride` bytes <-> a compact run (one row of `n` doubles)
    auto gather = [&](const double *src, double *dst, int n) -> cudaError_t {
        if (n == 0) return cudaSuccess;
        const MemKind k = classify(src);
        const bool dev = k == MemKind::Device || k == MemKind::Managed;
        return cudaMemcpy2DAsync(dst, 8, src, stride, 8, n, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                 s);
    };
    auto scatter = [&](const double *src, double *dst, int n) -> cudaError_t {
        if (n == 0) return cudaSuccess;
        const MemKind k = classify(dst);
        const bool dev = k == MemKind::Device || k == MemKind::Managed;
        return cudaMemcpy2DAsync(dst, stride, src, 8, 8, n, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                 s);
    };
    if (!inverse) {
        CK(gather(a, x, N));
        CK(line_d(false, x, N, wavelet, static_cast<double *>(tmp.p), s));
        CK(scatter(x, c_l, nl));
        CK(scatter(x + nl, h_out, nh));
    } else {
        CK(gather(a, x, nl));
        CK(gather(b, x + nl, nh));
        CK(line_d(true, x, N, wavelet, static_cast<double *>(tmp.p), s));
        CK(scatter(x, c_l, N));
    }
    return set_error(lane_finish(c));
}

// ------------------------------------------- strided 1D: combined calls
//
// The reference's callers transform banks of signals as loops of one
// dwt_cdf97_f_ex_stride_s call per signal, often from several OpenMP threads
// at once (src/libdwt.c:5512-5557).  One call costs a few launches and a
// synchronisation, tens of microseconds, almost all of it fixed cost; so
// calls that arrive while other threads' batches are on the GPU are
// combined: a thread that finds fewer than combine_batches() batches running
// takes every pending call, gathers their samples into the rows of one frame
// (the rows' addresses travel as kernel parameters), transforms all rows in
// one launch per (wavelet, direction, length) and scatters the results, and
// the calls it took return once that has synchronised.  A thread calling
// alone gets a batch of one.  Only calls whose memory the kernels address
// directly are combined (device and managed memory, and pageable host memory
// where the GPU walks the host's page tables); the others take the per-call
// path below.  DWT_GPU_COMBINE_1D=0 turns combining off.
struct PendingCall {
    int wavelet;
    bool inverse;
    int N;
    CallRow row;
    int rc;
    bool done;
    std::condition_variable cv;  // the call's thread waits here (done, or asked to lead)
};

static std::mutex g_comb_mu;
static std::vector<PendingCall *> g_comb_pending;
static int g_comb_running = 0;  // batches in flight

// Batches in flight at once, each on its own lane (4; DWT_GPU_COMBINE_BATCHES,
// 1 .. 8): a thread whose call arrives while the limit is reached waits for
// one to finish, then takes every queued call.  16 threads calling from an
// OpenMP loop, device memory: 76 / 74 / 72 us per call and thread with 2 / 3
// / 4 batches.
static int combine_batches()
{
    static const int n = [] {
        const char *e = getenv("DWT_GPU_COMBINE_BATCHES");
        const int v = e ? atoi(e) : 0;
        return v >= 1 && v <= 8 ? v : 4;
    }();
    return n;
}

static bool combine_enabled()
{
    static const bool on = [] {
        const char *v = getenv("DWT_GPU_COMBINE_1D");
        return !(v && v[0] == '0');
    }();
    return on;
}

// The kind of p and, for CUDA allocations (device, managed, pinned), the
// allocation holding it, [lo, hi): one driver query, so that the other
// pointers of a call that fall in the same allocation need none.  Memory the
// driver does not know is pageable host memory (as classify has it).
static MemKind classify_range(const void *p, uintptr_t &lo, uintptr_t &hi)
{
    using Fn = CUresult (*)(unsigned int, CUpointer_attribute *, void **, CUdeviceptr);
    static const Fn fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttributes", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        cudaGetLastError();
        return reinterpret_cast<Fn>(f);
    }();
    lo = hi = 0;
    if (!fn) return classify(p);
    unsigned int type = 0;
    int managed = 0;
    CUdeviceptr start = 0;
    size_t size = 0;
    CUpointer_attribute attrs[4] = {CU_POINTER_ATTRIBUTE_MEMORY_TYPE, CU_POINTER_ATTRIBUTE_IS_MANAGED,
                                    CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, CU_POINTER_ATTRIBUTE_RANGE_SIZE};
    void *vals[4] = {&type, &managed, &start, &size};
    if (fn(4, attrs, vals, reinterpret_cast<CUdeviceptr>(p)) != CUDA_SUCCESS || type == 0) return MemKind::Pageable;
    if (size > 0) {
        lo = uintptr_t(start);
        hi = lo + size;
    }
    if (managed || type == CU_MEMORYTYPE_UNIFIED) return MemKind::Managed;
    return type == CU_MEMORYTYPE_DEVICE ? MemKind::Device : MemKind::Pinned;
}

static bool reaches(MemKind k)
{
    return k == MemKind::Device || k == MemKind::Managed || (k == MemKind::Pageable && pageable_direct());
}

// Whether the kernels address every given pointer (nulls and repeats
// skipped), with one driver query per distinct CUDA allocation.
static bool kernel_reaches_all(const void *first, std::initializer_list<const void *> others)
{
    uintptr_t lo = 0, hi = 0;
    if (!reaches(classify_range(first, lo, hi))) return false;
    for (const void *q : others) {
        if (!q || q == first) continue;
        const uintptr_t u = reinterpret_cast<uintptr_t>(q);
        if (u >= lo && u < hi) continue;
        uintptr_t l2, h2;
        if (!reaches(classify_range(q, l2, h2))) return false;
    }
    return true;
}

// One (wavelet, direction, length) group of combined calls: gather, one
// launch over all rows, scatter, synchronise.
static int run_1d_rows(int wavelet, bool inverse, int N, PendingCall *const *calls, int n)
{
    if (n > 65535) return set_error(DWT_GPU_EINVAL);
    LaneGuard lane_guard(ctx());
    Lane &c = lane_guard.get();
    cudaStream_t s = c.stream;
    const int nl = (N + 1) / 2;
    const int nl4 = int(align_up(nl, 4));
    const long long P = align_up(N + 4, 32);
    std::vector<CallRow> rows(n);
    for (int k = 0; k < n; ++k) rows[k] = calls[k]->row;
    // up to kCallRowsParam rows travel as kernel parameters, more as a device array
    Buf desc;
    const CallRow *d_rows = nullptr;
    if (n > kCallRowsParam) {
        if (!desc.alloc(sizeof(CallRow) * n + 256, s)) return set_error(DWT_GPU_ENOMEM);
        CK(cudaMemcpyAsync(desc.p, rows.data(), sizeof(CallRow) * n, cudaMemcpyHostToDevice, s));
        d_rows = static_cast<const CallRow *>(desc.p);
    }
    if (N <= kCalls1dMaxN) {
        // one launch: gather, lift and scatter per call in shared memory
        CK(launch_calls_1d(d_rows, rows.data(), n, N, wavelet, inverse, s));
        return set_error(lane_finish(c));
    }
    Buf in(size_t(P) * n * 4 + 256, s), out(size_t(P) * n * 4 + 256, s);
    if (!in.p || !out.p) return set_error(DWT_GPU_ENOMEM);
    CK(launch_gather_calls(d_rows, rows.data(), n, N, inverse, in.f(), P, nl4, s));
    LevelDesc d{};
    d.w = N;
    d.h = n;
    d.rows_only = 1;
    d.in[0] = in.f();
    d.in_pitch[0] = P;
    if (inverse) {
        d.in[1] = in.f() + nl4;
        d.in_pitch[1] = P;
    }
    d.out[0] = out.f();
    d.out_pitch[0] = P;
    if (!inverse) {
        d.out[1] = out.f() + nl;
        d.out_pitch[1] = P;
    }
    plan_level(d, 0, inverse);
    CK(launch_level(d, wavelet, inverse, s, c.d_err));
    CK(launch_scatter_calls(d_rows, rows.data(), n, N, inverse, out.f(), P, s));
    return set_error(lane_finish(c));
}

static void run_combined(std::vector<PendingCall *> &batch)
{
    std::stable_sort(batch.begin(), batch.end(), [](const PendingCall *x, const PendingCall *y) {
        if (x->wavelet != y->wavelet) return x->wavelet < y->wavelet;
        if (x->inverse != y->inverse) return x->inverse < y->inverse;
        return x->N < y->N;
    });
    for (size_t i = 0; i < batch.size();) {
        size_t j = i + 1;
        while (j < batch.size() && batch[j]->wavelet == batch[i]->wavelet && batch[j]->inverse == batch[i]->inverse &&
               batch[j]->N == batch[i]->N)
            ++j;
        const int rc = run_1d_rows(batch[i]->wavelet, batch[i]->inverse, batch[i]->N, batch.data() + i, int(j - i));
        for (size_t k = i; k < j; ++k) batch[k]->rc = rc;
        i = j;
    }
}

// Queues the call and returns when a batch holding it completed (running
// that batch itself when none is running).
static int run_1d_combined(PendingCall &me)
{
    std::unique_lock<std::mutex> lk(g_comb_mu);
    g_comb_pending.push_back(&me);
    while (!me.done) {
        if (g_comb_running < combine_batches() && !g_comb_pending.empty()) {
            ++g_comb_running;
            std::vector<PendingCall *> batch;
            batch.swap(g_comb_pending);
            lk.unlock();
            run_combined(batch);
            lk.lock();
            --g_comb_running;
            // wake exactly the calls of the batch, and one queued call to
            // lead the next batch (no herd of waiters on one variable)
            for (PendingCall *q : batch) {
                q->done = true;
                if (q != &me) q->cv.notify_one();
            }
            if (!g_comb_pending.empty()) g_comb_pending.front()->cv.notify_one();
        } else {
            me.cv.wait(lk);
        }
    }
    return me.rc;
}

int run_1d(int wavelet, bool inverse, const float *a, const float *b, float *c_l, float *h_out, int N,
           int stride)
{
    t_last_error = DWT_GPU_OK;
    if (N < 0 || stride == 0) {
        log_error("invalid 1D arguments (N=%d, stride=%d)\n", N, stride);
        return set_error(DWT_GPU_EINVAL);
    }
    if (N == 0) return DWT_GPU_OK;
    if (stride < 4) {
        log_error("stride %d smaller than a sample\n", stride);
        return set_error(DWT_GPU_EINVAL);
    }
    if (!a || !c_l || (inverse && N / 2 > 0 && !b) || (!inverse && N / 2 > 0 && !h_out)) {
        log_error("null 1D signal pointer\n");
        return set_error(DWT_GPU_EINVAL);
    }
    if (combine_enabled()) {
        const int nh = N / 2;
        const bool reach = (!inverse || nh == 0 || b) && (inverse || nh == 0 || h_out) &&
                           kernel_reaches_all(a, {c_l, inverse && nh ? b : nullptr, !inverse && nh ? h_out : nullptr});
        if (reach) {
            PendingCall me{wavelet, inverse, N, CallRow{a, b, c_l, h_out, stride}, DWT_GPU_OK, false, {}};
            return set_error(run_1d_combined(me));
        }
    }
    const NvtxRange range("dwt 1D %s %s N=%d", wavelet == CDF97 ? "cdf97" : "cdf53", inverse ? "inverse" : "forward",
                          N);
    LaneGuard lane_guard(ctx());
    Lane &c = lane_guard.get();
    cudaStream_t s = c.stream;
    const int nl = (N + 1) / 2, nh = N / 2;
    const long long P = align_up(N, 32);
    Buf in(size_t(P) * 4 + 256, s), out(size_t(P) * 4 + 256, s);
    if (!in.p || !out.p) return set_error(DWT_GPU_ENOMEM);

    // stage the input samples into IN (forward: N samples; inverse: L then H);
    // the gather and scatter kernels address device memory and pageable host
    // memory the GPU reaches itself, the copy engines the rest
    auto kernel_reach = [](const void *p) {
        const MemKind k = classify(p);
        return k == MemKind::Device || k == MemKind::Managed || (k == MemKind::Pageable && pageable_direct());
    };
    auto gather = [&](const float *src, float *dst, int n) -> cudaError_t {
        if (n == 0) return cudaSuccess;
        if (kernel_reach(src)) return launch_gather_signals(src, n, stride, 1, 1, 0, 0, dst, P, s);
        return cudaMemcpy2DAsync(dst, 4, src, stride, 4, n, cudaMemcpyHostToDevice, s);
    };
    auto scatter = [&](const float *src, float *dst, int n) -> cudaError_t {
        if (n == 0) return cudaSuccess;
        if (kernel_reach(dst)) return launch_scatter_signals(src, P, n, dst, stride, 1, 1, 0, 0, s);
        return cudaMemcpy2DAsync(dst, stride, src, 4, 4, n, cudaMemcpyDeviceToHost, s);
    };

    LevelDesc d{};
    d.w = N;
    d.h = 1;
    d.rows_only = 1;
    if (!inverse) {
        CK(gather(a, in.f(), N));
        d.in[0] = in.f();
        d.in_pitch[0] = P;
        d.out[0] = out.f();
        d.out[1] = out.f() + nl;
        d.out_pitch[0] = d.out_pitch[1] = P;
    } else {
        // L at IN[0, nl), H at IN[nl4, ...) with nl4 16-byte aligned
        const int nl4 = int(align_up(nl, 4));
        CK(gather(a, in.f(), nl));
        CK(gather(b, in.f() + nl4, nh));
        d.in[0] = in.f();
        d.in[1] = in.f() + nl4;
        d.in_pitch[0] = d.in_pitch[1] = P;
        d.out[0] = out.f();
        d.out_pitch[0] = P;
    }
    plan_level(d, 0, inverse);
    CK(launch_level(d, wavelet, inverse, s, c.d_err));
    if (!inverse) {
        CK(scatter(out.f(), c_l, nl));
        CK(scatter(out.f() + nl, h_out, nh));
    } else {
        CK(scatter(out.f(), c_l, N));
    }
    return set_error(lane_finish(c));
}

// Batched strided 1D, in place: gather every signal into a row of IN,
// transform all rows in one launch, scatter back.
int run_1d_batch(int wavelet, bool inverse, void *base, int N, int stride, long long count, int group,
                 long long group_stride, int lane_stride)
{
    t_last_error = DWT_GPU_OK;
    if (N < 0 || stride < 4 || count < 0 || group <= 0 || !base) {
        log_error("invalid batched 1D arguments\n");
        return set_error(DWT_GPU_EINVAL);
    }
    if (N == 0 || count == 0) return DWT_GPU_OK;
    if (count > 0x7fffffffLL) return set_error(DWT_GPU_EINVAL);
    LaneGuard lane_guard(ctx());
    Lane &c = lane_guard.get();
    cudaStream_t s = c.stream;
    const MemKind kind = classify(base);
    const bool on_device = kind == MemKind::Device || kind == MemKind::Managed;
    const int nl = (N + 1) / 2;

    // the bank's byte span (for host memory)
    const long long last = (count - 1) / group * group_stride + (count - 1) % group * (long long)lane_stride;
    const long long sb = last + (long long)(N - 1) * stride + 4;

    // dense sample-interleaved groups: one CTA per group, in place
    if (count % group == 0 && signals_fast_ok(base, N, stride, group, group_stride, lane_stride)) {
        const long long groups = count / group;
        void *dev = base;
        Buf span;
        if (!on_device) {
            const long long gsb = (groups - 1) * group_stride + 4LL * N * group;
            if (!span.alloc(size_t(gsb) + 16, s)) return set_error(DWT_GPU_ENOMEM);
            CK(cudaMemcpyAsync(span.p, base, size_t(gsb), cudaMemcpyHostToDevice, s));
            dev = span.p;
        }
        CK(launch_signals(wavelet, inverse, static_cast<float *>(dev), N, group, group_stride, groups, s, c.sm_count,
                          c.d_err));
        if (!on_device)
            CK(cudaMemcpyAsync(base, span.p, size_t((groups - 1) * group_stride + 4LL * N * group),
                               cudaMemcpyDeviceToHost, s));
        return set_error(lane_finish(c));
    }

    const long long P = align_up(N + 4, 32);
    const int nl4 = int(align_up(nl, 4));
    Buf in(size_t(P) * count * 4 + 256, s), out(size_t(P) * count * 4 + 256, s);
    if (!in.p || !out.p) return set_error(DWT_GPU_ENOMEM);
    Buf span;
    const void *src = base;
    if (!on_device) {
        if (!span.alloc(size_t(sb) + 16, s)) return set_error(DWT_GPU_ENOMEM);
        CK(cudaMemcpyAsync(span.p, base, size_t(sb), cudaMemcpyHostToDevice, s));
        src = span.p;
    }
    LevelDesc d{};
    d.w = N;
    d.h = int(count);
    d.rows_only = 1;
    if (!inverse) {
        CK(launch_gather_signals(src, N, stride, count, group, group_stride, lane_stride, in.f(), P, s));
        d.in[0] = in.f();
        d.in_pitch[0] = P;
        d.out[0] = out.f();
        d.out[1] = out.f() + nl;
        d.out_pitch[0] = d.out_pitch[1] = P;
    } else {
        // L samples to columns [0, nl), H samples to [nl4, nl4 + N/2) of each row
        CK(launch_gather_signals(src, nl, stride, count, group, group_stride, lane_stride, in.f(), P, s));
        CK(launch_gather_signals(static_cast<const char *>(src) + (long long)nl * stride, N / 2, stride,
                                 count, group, group_stride, lane_stride, in.f() + nl4, P, s));
        d.in[0] = in.f();
        d.in[1] = in.f() + nl4;
        d.in_pitch[0] = d.in_pitch[1] = P;
        d.out[0] = out.f();
        d.out_pitch[0] = P;
    }
    plan_level(d, 0, inverse);
    CK(launch_level(d, wavelet, inverse, s, c.d_err));
    void *dst = on_device ? base : span.p;
    CK(launch_scatter_signals(out.f(), P, N, dst, stride, count, group, group_stride, lane_stride, s));
    if (!on_device) CK(cudaMemcpyAsync(base, span.p, size_t(sb), cudaMemcpyDeviceToHost, s));
    return set_error(lane_finish(c));
}

// Every channel of a dense interleaved float image in one call: one copy of
// the image each way, the channels split into compact planes, the level
// pipeline per plane, and interleaved back.  The same bits as the drop-in
// on each channel (ptr + 4c, stride_y = 4 * channels).
static int run_2d_channels(int wavelet, bool inverse, void *ptr, int stride_x, int channels, int w, int h,
                           int *j_levels, int decompose_one)
{
    t_last_error = DWT_GPU_OK;
    if (!ptr || !j_levels || channels < 1 || w < 0 || h < 0 || (long long)stride_x < 4LL * channels * w ||
        (reinterpret_cast<uintptr_t>(ptr) & 3) != 0) {
        log_error("invalid interleaved 2D arguments\n");
        return set_error(DWT_GPU_EINVAL);
    }
    const int lim = (decompose_one ? std::max(w, h) : std::min(w, h)) > 0
                        ? ceil_log2_int(decompose_one ? std::max(w, h) : std::min(w, h))
                        : 0;
    int J;
    if (!inverse) {
        if (*j_levels < 0 || *j_levels > lim) *j_levels = lim;
        J = *j_levels;
    } else {
        J = (*j_levels < 0 || *j_levels > lim) ? lim : *j_levels;
    }
    if (J == 0 || w == 0 || h == 0) return DWT_GPU_OK;
    LaneGuard lane_guard(ctx());
    Lane &c = lane_guard.get();
    cudaStream_t s = c.stream;
    const MemKind kind = classify(ptr);
    const bool on_device = kind == MemKind::Device || kind == MemKind::Managed;
    const long long rowb = 4LL * channels * w;
    const long long P = align_up(w, 32);
    const long long plane = P * h + 64;
    Buf stage, in(size_t(plane) * channels * 4 + 256, s), out(size_t(plane) * channels * 4 + 256, s);
    if (!in.p || !out.p) return set_error(DWT_GPU_ENOMEM);
    const void *src = ptr;
    long long src_pitch = stride_x;
    if (!on_device) {
        if (!stage.alloc(size_t(rowb) * h + 256, s)) return set_error(DWT_GPU_ENOMEM);
        CK(cudaMemcpy2DAsync(stage.p, rowb, ptr, stride_x, rowb, h, cudaMemcpyHostToDevice, s));
        src = stage.p;
        src_pitch = rowb;
    }
    CK(launch_deinterleave(src, src_pitch, channels, w, h, in.f(), P, plane, s));
    long long p0, p1;
    const size_t sf = dense_scratch_floats(w, h, J, &p0, &p1);
    Buf scratch(sf * 4 + 256, s);
    if (sf && !scratch.p) return set_error(DWT_GPU_ENOMEM);
    for (int ch = 0; ch < channels; ++ch) {
        const float *pin = in.f() + ch * plane;
        float *pout = out.f() + ch * plane;
        if (!inverse)
            CK(dense_forward(pin, P, pout, P, w, h, J, wavelet, scratch.f(), s, c.d_err, 0));
        else
            CK(dense_inverse(pin, P, pout, P, w, h, J, wavelet, scratch.f(), s, c.d_err, 0));
    }
    if (!on_device) {
        CK(launch_interleave(out.f(), P, plane, channels, w, h, stage.p, rowb, s));
        CK(cudaMemcpy2DAsync(ptr, stride_x, stage.p, rowb, rowb, h, cudaMemcpyDeviceToHost, s));
    } else {
        CK(launch_interleave(out.f(), P, plane, channels, w, h, ptr, stride_x, s));
    }
    return set_error(lane_finish(c));
}

int run_2d_dev(int wavelet, bool inverse, const float *src, long long src_pitch_bytes, float *dst,
               long long dst_pitch_bytes, int w, int h, int j_levels, int decompose_one, cudaStream_t s)
{
    t_last_error = DWT_GPU_OK;
    if (w <= 0 || h <= 0 || !src || !dst || (src_pitch_bytes % 16) != 0 ||
        (reinterpret_cast<uintptr_t>(src) & 15) != 0 || (dst_pitch_bytes % 4) != 0 ||
        src_pitch_bytes < 4LL * w || dst_pitch_bytes < 4LL * w) {
        log_error("invalid device 2D arguments\n");
        return set_error(DWT_GPU_EINVAL);
    }
    const int lim = ceil_log2_int(decompose_one ? std::max(w, h) : std::min(w, h));
    const int J = (j_levels < 0 || j_levels > lim) ? lim : j_levels;
    if (J == 0) {
        if (src != dst)
            CK(cudaMemcpy2DAsync(dst, dst_pitch_bytes, src, src_pitch_bytes, size_t(w) * 4, h,
                                 cudaMemcpyDeviceToDevice, s));
        return 0;
    }
    if (frames_overlap(src, src_pitch_bytes, dst, dst_pitch_bytes, w, h)) {
        log_error("dwt_gpu_2_dev: the source and destination frames overlap (out of place only)\n");
        return set_error(DWT_GPU_EINVAL);
    }
    const NvtxRange range("dwt 2D device %s %s %dx%d j=%d", wavelet == CDF97 ? "cdf97" : "cdf53",
                          inverse ? "inverse" : "forward", w, h, J);
    Context &c = ctx();
    long long p0, p1;
    const size_t sf = dense_scratch_floats(w, h, J, &p0, &p1);
    void *scratch = sf ? c.pool.alloc(sf * 4 + 256, s) : nullptr;
    if (sf && !scratch) return set_error(DWT_GPU_ENOMEM);
    cudaError_t e = inverse ? dense_inverse(src, src_pitch_bytes / 4, dst, dst_pitch_bytes / 4, w, h, J,
                                            wavelet, static_cast<float *>(scratch), s, c.d_err, 0)
                            : dense_forward(src, src_pitch_bytes / 4, dst, dst_pitch_bytes / 4, w, h, J,
                                            wavelet, static_cast<float *>(scratch), s, c.d_err, 0);
    if (scratch) c.pool.release(scratch, s);
    if (e != cudaSuccess) {
        log_error("CUDA error %s\n", cudaGetErrorString(e));
        return set_error(DWT_GPU_ECUDA);
    }
    return J;
}

// Failure detection, exercised without a fault: one warp waits on an
// mbarrier that nothing completes, through the bounded wait the level kernels
// use, with a short limit.  The wait gives up, the error word is set and the
// kernel returns normally.
__global__ void wait_timeout_kernel(uint32_t iterations, int *err)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncwarp();
    const bool done = mbar_wait_bounded(&bar, 0, iterations);  // no arrival is ever made
    if (!__all_sync(0xffffffffu, done) && threadIdx.x == 0) atomicCAS(err, 0, int(kErrWaitTimeout));
}

cudaError_t launch_wait_timeout(uint32_t iterations, int *err, cudaStream_t s)
{
    wait_timeout_kernel<<<1, 32, 0, s>>>(iterations, err);
    return cudaGetLastError();
}

}  // namespace dwt

using namespace dwt;

// ====================================================================== C ABI

static void die_if(int rc)
{
    if (rc != DWT_GPU_OK) {
        log_error("libdwt_gb300: %s\n", dwt_gpu_error_string(rc));
        abort();  // the reference's fatal-error convention (src/libdwt.c:7512-7530)
    }
}

extern "C" {

int dwt_gpu_get_last_error(void) { return t_last_error; }

const char *dwt_gpu_error_string(int code)
{
    switch (code) {
    case DWT_GPU_OK: return "success";
    case DWT_GPU_EINVAL: return "invalid argument";
    case DWT_GPU_ECUDA: return "CUDA error";
    case DWT_GPU_ENOMEM: return "out of device memory";
    case DWT_GPU_EDEVICE: return "device-side wait gave up";
    case DWT_GPU_EBUSY: return "admission refused";
    case DWT_GPU_ENOTFOUND: return "unknown request";
    default: return "unknown error";
    }
}

int dwt_gpu_2f_s(int wavelet, void *ptr, int stride_x, int stride_y, int ox, int oy, int ix, int iy,
                 int *j_max_ptr, int decompose_one, int zero_padding)
{
    if (!j_max_ptr || (wavelet != CDF97 && wavelet != CDF53)) return set_error(DWT_GPU_EINVAL);
    return run_2d(wavelet, false, ptr, stride_x, stride_y, ox, oy, ix, iy, j_max_ptr, 0, decompose_one,
                  zero_padding);
}

int dwt_gpu_2i_s(int wavelet, void *ptr, int stride_x, int stride_y, int ox, int oy, int ix, int iy,
                 int j_max, int decompose_one, int zero_padding)
{
    if (wavelet != CDF97 && wavelet != CDF53) return set_error(DWT_GPU_EINVAL);
    return run_2d(wavelet, true, ptr, stride_x, stride_y, ox, oy, ix, iy, nullptr, j_max, decompose_one,
                  zero_padding);
}

int dwt_gpu_1_s(int wavelet, int inverse, const float *a, const float *b, float *c_or_l, float *h_or_null,
                int N, int stride)
{
    if (wavelet != CDF97 && wavelet != CDF53) return set_error(DWT_GPU_EINVAL);
    return run_1d(wavelet, inverse != 0, a, b, c_or_l, h_or_null, N, stride);
}

int dwt_gpu_2_channels_s(int wavelet, int inverse, void *ptr, int stride_x, int channels, int w, int h,
                         int *j_levels, int decompose_one)
{
    if (wavelet != CDF97 && wavelet != CDF53) return set_error(DWT_GPU_EINVAL);
    return run_2d_channels(wavelet, inverse != 0, ptr, stride_x, channels, w, h, j_levels, decompose_one);
}

int dwt_gpu_2f_d(int wavelet, void *ptr, int stride_x, int stride_y, int ox, int oy, int ix, int iy,
                 int *j_max_ptr, int decompose_one, int zero_padding)
{
    if (!j_max_ptr || (wavelet != CDF97 && wavelet != CDF53)) return set_error(DWT_GPU_EINVAL);
    return run_2d_d(wavelet, false, ptr, stride_x, stride_y, ox, oy, ix, iy, j_max_ptr, 0, decompose_one,
                    zero_padding);
}

int dwt_gpu_2i_d(int wavelet, void *ptr, int stride_x, int stride_y, int ox, int oy, int ix, int iy,
                 int j_max, int decompose_one, int zero_padding)
{
    if (wavelet != CDF97 && wavelet != CDF53) return set_error(DWT_GPU_EINVAL);
    return run_2d_d(wavelet, true, ptr, stride_x, stride_y, ox, oy, ix, iy, nullptr, j_max, decompose_one,
                    zero_padding);
}

int dwt_gpu_1_d(int wavelet, int inverse, const double *a, const double *b, double *c_or_l, double *h_or_null,
                int N, int stride)
{
    if (wavelet != CDF97 && wavelet != CDF53) return set_error(DWT_GPU_EINVAL);
    return run_1d_d(wavelet, inverse != 0, a, b, c_or_l, h_or_null, N, stride);
}

int dwt_gpu_2_dev(int wavelet, int inverse, const float *src, long long src_pitch_bytes, float *dst,
                  long long dst_pitch_bytes, int w, int h, int j_levels, int decompose_one, void *stream)
{
    if (wavelet != CDF97 && wavelet != CDF53) return set_error(DWT_GPU_EINVAL);
    return run_2d_dev(wavelet, inverse != 0, src, src_pitch_bytes, dst, dst_pitch_bytes, w, h, j_levels,
                      decompose_one, static_cast<cudaStream_t>(stream));
}

int dwt_gpu_1_batch_s(int wavelet, int inverse, void *base, int N, int stride, long long count, int group,
                      long long group_stride, int lane_stride)
{
    if (wavelet != CDF97 && wavelet != CDF53) return set_error(DWT_GPU_EINVAL);
    return run_1d_batch(wavelet, inverse != 0, base, N, stride, count, group, group_stride, lane_stride);
}

int dwt_gpu_level_dev(int wavelet, int inverse, int w, int h, const float *const in[4],
                      const long long in_pitch_bytes[4], float *const out[4],
                      const long long out_pitch_bytes[4], void *stream)
{
    t_last_error = DWT_GPU_OK;
    if ((wavelet != CDF97 && wavelet != CDF53) || w <= 0 || h <= 0 || !in || !out)
        return set_error(DWT_GPU_EINVAL);
    LevelDesc d{};
    d.w = w;
    d.h = h;
    const int nin = inverse ? 4 : 1, nout = inverse ? 1 : 4;
    for (int k = 0; k < nin; ++k) {
        if (!in[k] || (in_pitch_bytes[k] % 16) != 0) return set_error(DWT_GPU_EINVAL);
        d.in[k] = in[k];
        d.in_pitch[k] = in_pitch_bytes[k] / 4;
    }
    if (!inverse && (reinterpret_cast<uintptr_t>(in[0]) & 15) != 0) return set_error(DWT_GPU_EINVAL);
    for (int k = 0; k < nout; ++k) {
        if (!out[k] || (out_pitch_bytes[k] % 4) != 0) return set_error(DWT_GPU_EINVAL);
        d.out[k] = out[k];
        d.out_pitch[k] = out_pitch_bytes[k] / 4;
    }
    plan_level(d, 0, inverse != 0);
    Context &c = ctx();
    cudaError_t e = launch_level(d, wavelet, inverse != 0, static_cast<cudaStream_t>(stream), c.d_err);
    if (e != cudaSuccess) {
        log_error("CUDA error %s\n", cudaGetErrorString(e));
        return set_error(DWT_GPU_ECUDA);
    }
    return DWT_GPU_OK;
}

int dwt_gpu_dense_launches(int w, int h, int j_levels)
{
    if (w <= 0 || h <= 0) return set_error(DWT_GPU_EINVAL);
    const int J = j_levels < 0 ? ceil_log2_int(std::min(w, h)) : j_levels;
    if (J == 0) return 0;
    const int j0 = coarse_level(w, h, J);
    return j0 + (j0 < J ? 1 : 0);
}

int dwt_gpu_selftest_wait_timeout(int iterations)
{
    t_last_error = DWT_GPU_OK;
    if (iterations <= 0) return set_error(DWT_GPU_EINVAL);
    LaneGuard lane_guard(ctx());
    Lane &c = lane_guard.get();
    wait_timeout_kernel<<<1, 32, 0, c.stream>>>(uint32_t(iterations), c.d_err);
    CK(cudaGetLastError());
    return set_error(lane_finish(c));
}

int dwt_gpu_selftest_inplace_wait_timeout(int iterations)
{
    t_last_error = DWT_GPU_OK;
    if (iterations <= 0) return set_error(DWT_GPU_EINVAL);
    LaneGuard lane_guard(ctx());
    Lane &c = lane_guard.get();
    const size_t bytes = size_t(order_wait_timeout_words()) * 4;
    Buf order(bytes, c.stream);
    if (!order.p) return set_error(DWT_GPU_ENOMEM);
    CK(cudaMemsetAsync(order.p, 0, bytes, c.stream));
    CK(launch_order_wait_timeout(uint32_t(iterations), static_cast<int *>(order.p), c.d_err, c.stream));
    return set_error(lane_finish(c));
}

int dwt_gpu_inplace_plan(int wavelet, int inverse, int w, int h, int detail_row, int *seg_pairs, int *n_segs,
                         int *stage_seg, int *readers)
{
    t_last_error = DWT_GPU_OK;
    if ((wavelet != CDF97 && wavelet != CDF53) || w < 2 || h < 2 || !seg_pairs || !n_segs || !stage_seg ||
        (detail_row >= 0 && detail_row < (h + 1) / 2))
        return set_error(DWT_GPU_EINVAL);
    LevelDesc d{};
    d.w = w;
    d.h = h;
    plan_level(d, 0, inverse != 0);
    const int lat = wavelet == CDF97 ? 2 : 1;
    *seg_pairs = d.seg_pairs;
    *n_segs = d.n_segs;
    const int dy = detail_row < 0 ? (h + 1) / 2 : detail_row;
    *stage_seg = inplace_stage_seg(h, d.seg_pairs, d.n_segs, lat, inverse != 0, inplace_lead(), dy);
    if (readers)
        for (int s = 0; s < d.n_segs; ++s)
            inplace_readers(h, d.seg_pairs, d.n_segs, lat, inverse != 0, s, *stage_seg, dy, readers[2 * s],
                            readers[2 * s + 1]);
    return DWT_GPU_OK;
}

int dwt_gpu_sync_check(void)
{
    // the pooled context is only checked when it exists: a caller of the
    // allocation-free entry point must be able to check its work without
    // having the context (and its allocations) created
    Context *c = nullptr;
    {
        std::lock_guard<std::mutex> g(g_init_mu);
        c = g_ctx;
        if (c) cudaSetDevice(c->device);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return set_error(DWT_GPU_ECUDA);
    const int rc_noalloc = noalloc_device_error();
    const int rc_ctx = c ? check_device_error(*c) : DWT_GPU_OK;
    return set_error(rc_ctx != DWT_GPU_OK ? rc_ctx : rc_noalloc);
}

void dwt_cdf97_2f_s(void *ptr, int stride_x, int stride_y, int ox, int oy, int ix, int iy, int *j_max_ptr,
                    int decompose_one, int zero_padding)
{
    die_if(dwt_gpu_2f_s(CDF97, ptr, stride_x, stride_y, ox, oy, ix, iy, j_max_ptr, decompose_one, zero_padding));
}

void dwt_cdf53_2f_s(void *ptr, int stride_x, int stride_y, int ox, int oy, int ix, int iy, int *j_max_ptr,
                    int decompose_one, int zero_padding)
{
    die_if(dwt_gpu_2f_s(CDF53, ptr, stride_x, stride_y, ox, oy, ix, iy, j_max_ptr, decompose_one, zero_padding));
}

void dwt_cdf97_2i_s(void *ptr, int stride_x, int stride_y, int ox, int oy, int ix, int iy, int j_max,
                    int decompose_one, int zero_padding)
{
    die_if(dwt_gpu_2i_s(CDF97, ptr, stride_x, stride_y, ox, oy, ix, iy, j_max, decompose_one, zero_padding));
}

void dwt_cdf53_2i_s(void *ptr, int stride_x, int stride_y, int ox, int oy, int ix, int iy, int j_max,
                    int decompose_one, int zero_padding)
{
    die_if(dwt_gpu_2i_s(CDF53, ptr, stride_x, stride_y, ox, oy, ix, iy, j_max, decompose_one, zero_padding));
}

void dwt_cdf97_f_ex_stride_s(const float *src, float *dst_l, float *dst_h, float *tmp, int N, int stride)
{
    (void)tmp;
    die_if(run_1d(CDF97, false, src, nullptr, dst_l, dst_h, N, stride));
}

void dwt_cdf97_i_ex_stride_s(const float *src_l, const float *src_h, float *dst, float *tmp, int N, int stride)
{
    (void)tmp;
    die_if(run_1d(CDF97, true, src_l, src_h, dst, nullptr, N, stride));
}

void dwt_cdf53_f_ex_stride_s(const float *src, float *dst_l, float *dst_h, float *tmp, int N, int stride)
{
    (void)tmp;
    die_if(run_1d(CDF53, false, src, nullptr, dst_l, dst_h, N, stride));
}

void dwt_cdf53_i_ex_stride_s(const float *src_l, const float *src_h, float *dst, float *tmp, int N, int stride)
{
    (void)tmp;
    die_if(run_1d(CDF53, true, src_l, src_h, dst, nullptr, N, stride));
}

void dwt_cdf97_f_ex_s(const float *src, float *dst_l, float *dst_h, float *tmp, int N)
{
    dwt_cdf97_f_ex_stride_s(src, dst_l, dst_h, tmp, N, sizeof(float));
}

void dwt_cdf53_f_ex_s(const float *src, float *dst_l, float *dst_h, float *tmp, int N)
{
    dwt_cdf53_f_ex_stride_s(src, dst_l, dst_h, tmp, N, sizeof(float));
}

void dwt_cdf97_i_ex_s(const float *src_l, const float *src_h, float *dst, float *tmp, int N)
{
    dwt_cdf97_i_ex_stride_s(src_l, src_h, dst, tmp, N, sizeof(float));
}

void dwt_cdf53_i_ex_s(const float *src_l, const float *src_h, float *dst, float *tmp, int N)
{
    dwt_cdf53_i_ex_stride_s(src_l, src_h, dst, tmp, N, sizeof(float));
}

void dwt_cdf97_f_s(const float *src, float *dst, float *tmp, int N)
{
    dwt_cdf97_f_ex_s(src, dst, dst + (N + 1) / 2, tmp, N);
}

void dwt_cdf53_f_s(const float *src, float *dst, float *tmp, int N)
{
    dwt_cdf53_f_ex_s(src, dst, dst + (N + 1) / 2, tmp, N);
}

void dwt_cdf97_i_s(const float *src, float *dst, float *tmp, int N)
{
    dwt_cdf97_i_ex_s(src, src + (N + 1) / 2, dst, tmp, N);
}

void dwt_cdf53_i_s(const float *src, float *dst, float *tmp, int N)
{
    dwt_cdf53_i_ex_s(src, src + (N + 1) / 2, dst, tmp, N);
}

// ------------------------------------------------ double precision (_d)

void dwt_cdf97_2f_d(void *ptr, int stride_x, int stride_y, int ox, int oy, int ix, int iy, int *j_max_ptr,
                    int decompose_one, int zero_padding)
{
    die_if(dwt_gpu_2f_d(CDF97, ptr, stride_x, stride_y, ox, oy, ix, iy, j_max_ptr, decompose_one, zero_padding));
}

void dwt_cdf53_2f_d(void *ptr, int stride_x, int stride_y, int ox, int oy, int ix, int iy, int *j_max_ptr,
                    int decompose_one, int zero_padding)
{
    die_if(dwt_gpu_2f_d(CDF53, ptr, stride_x, stride_y, ox, oy, ix, iy, j_max_ptr, decompose_one, zero_padding));
}

void dwt_cdf97_2i_d(void *ptr, int stride_x, int stride_y, int ox, int oy, int ix, int iy, int j_max,
                    int decompose_one, int zero_padding)
{
    die_if(dwt_gpu_2i_d(CDF97, ptr, stride_x, stride_y, ox, oy, ix, iy, j_max, decompose_one, zero_padding));
}

void dwt_cdf53_2i_d(void *ptr, int stride_x, int stride_y, int ox, int oy, int ix, int iy, int j_max,
                    int decompose_one, int zero_padding)
{
    die_if(dwt_gpu_2i_d(CDF53, ptr, stride_x, stride_y, ox, oy, ix, iy, j_max, decompose_one, zero_padding));
}

void dwt_cdf97_f_ex_stride_d(const double *src, double *dst_l, double *dst_h, double *tmp, int N, int stride)
{
    (void)tmp;
    die_if(run_1d_d(CDF97, false, src, nullptr, dst_l, dst_h, N, stride));
}

void dwt_cdf97_i_ex_stride_d(const double *src_l, const double *src_h, double *dst, double *tmp, int N,
                             int stride)
{
    (void)tmp;
    die_if(run_1d_d(CDF97, true, src_l, src_h, dst, nullptr, N, stride));
}

void dwt_cdf53_f_ex_stride_d(const double *src, double *dst_l, double *dst_h, double *tmp, int N, int stride)
{
    (void)tmp;
    die_if(run_1d_d(CDF53, false, src, nullptr, dst_l, dst_h, N, stride));
}

void dwt_cdf53_i_ex_stride_d(const double *src_l, const double *src_h, double *dst, double *tmp, int N,
                             int stride)
{
    (void)tmp;
    die_if(run_1d_d(CDF53, true, src_l, src_h, dst, nullptr, N, stride));
}

void dwt_cdf97_f_ex_d(const double *src, double *dst_l, double *dst_h, double *tmp, int N)
{
    dwt_cdf97_f_ex_stride_d(src, dst_l, dst_h, tmp, N, sizeof(double));
}

void dwt_cdf53_f_ex_d(const double *src, double *dst_l, double *dst_h, double *tmp, int N)
{
    dwt_cdf53_f_ex_stride_d(src, dst_l, dst_h, tmp, N, sizeof(double));
}

void dwt_cdf97_i_ex_d(const double *src_l, const double *src_h, double *dst, double *tmp, int N)
{
    dwt_cdf97_i_ex_stride_d(src_l, src_h, dst, tmp, N, sizeof(double));
}

void dwt_cdf53_i_ex_d(const double *src_l, const double *src_h, double *dst, double *tmp, int N)
{
    dwt_cdf53_i_ex_stride_d(src_l, src_h, dst, tmp, N, sizeof(double));
}

void dwt_cdf97_f_d(const double *src, double *dst, double *tmp, int N)
{
    dwt_cdf97_f_ex_d(src, dst, dst + (N + 1) / 2, tmp, N);
}

void dwt_cdf53_f_d(const double *src, double *dst, double *tmp, int N)
{
    dwt_cdf53_f_ex_d(src, dst, dst + (N + 1) / 2, tmp, N);
}

void dwt_cdf97_i_d(const double *src, double *dst, double *tmp, int N)
{
    dwt_cdf97_i_ex_d(src, src + (N + 1) / 2, dst, tmp, N);
}

void dwt_cdf53_i_d(const double *src, double *dst, double *tmp, int N)
{
    dwt_cdf53_i_ex_d(src, src + (N + 1) / 2, dst, tmp, N);
}

void dwt_util_init(void) { (void)ctx(); }

void dwt_util_finish(void) { ctx_finish(); }

void dwt_util_set_accel(int accel_type) { g_accel.store(accel_type); }

int dwt_util_ceil_log2(int x) { return ceil_log2_int(x); }

int dwt_util_pow2_ceil_log2(int x) { return 1 << ceil_log2_int(x); }

}  // extern "C"
