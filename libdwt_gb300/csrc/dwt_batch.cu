// Batched 2D transforms: thousands of images of uneven sizes, mixed wavelets
// and directions, in one persistent launch replayed as a CUDA graph.
//
// Work is cut into items: the warp units of every level of every image (a
// strip of 120 output columns by a segment of row pairs, as in the per-level
// kernel) and, per image, one "tail" item in which a single warp runs all the
// remaining small levels in its shared memory (the levels whose band fits
// tail_side x tail_side; the fused-level depth).  Items are ordered by phase
// (forward: level 0 units of all images, then level 1, ..., then the tails;
// inverse: tails first, then levels from coarse to fine) and handed out by an
// atomic ticket.  An item of phase p of image i waits for all items of phase
// p-1 of image i (a per-image, per-phase completion counter).  A warp waits
// only for items with smaller tickets, which were handed to warps that never
// wait for it, so the wait always ends; it is bounded anyway and raises the
// device error word if it gives up.
//
// The segment length (tile height), the tail side (fused-level depth) and the
// number of resident CTAs per SM are chosen by the autotuner in this file:
// it times candidate settings on the batch itself and caches the winner per
// batch signature in a text file.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/libdwt.h"
#include "dwt_batch.cuh"
#include "dwt_capi_internal.h"
#include "dwt_recur.cuh"
#include "dwt_units.cuh"

namespace dwt {

namespace {

// The level descriptor of forward level j (LL_j -> LL_{j+1} + details) or of
// inverse level j (LL_j + details -> LL_{j-1}) of image I.
__device__ LevelDesc level_desc(const BatchImage &I, int j)
{
    LevelDesc d{};
    if (!I.inverse) {
        const int w = ceil_div_pow2(I.w, j), h = ceil_div_pow2(I.h, j);
        const int wd = (w + 1) >> 1, hd = (h + 1) >> 1;
        d.w = w;
        d.h = h;
        d.in[0] = j == 0 ? I.src : I.ll[(j - 1) & 1];
        d.in_pitch[0] = j == 0 ? I.src_pitch : I.llp[(j - 1) & 1];
        if (j == I.J - 1) {
            d.out[0] = I.dst;
            d.out_pitch[0] = I.dst_pitch;
        } else {
            d.out[0] = I.ll[j & 1];
            d.out_pitch[0] = I.llp[j & 1];
        }
        d.out[1] = I.dst + wd;
        d.out[2] = I.dst + hd * I.dst_pitch;
        d.out[3] = I.dst + hd * I.dst_pitch + wd;
        d.out_pitch[1] = d.out_pitch[2] = d.out_pitch[3] = I.dst_pitch;
        d.n_strips = I.n_strips[j];
        d.seg_pairs = I.seg[j];
        d.n_segs = I.n_segs[j];
    } else {
        const int w = ceil_div_pow2(I.w, j - 1), h = ceil_div_pow2(I.h, j - 1);
        const int ws = (w + 1) >> 1, hs = (h + 1) >> 1;
        d.w = w;
        d.h = h;
        d.in[0] = j == I.J ? I.src : I.ll[(j - 1) & 1];
        d.in_pitch[0] = j == I.J ? I.src_pitch : I.llp[(j - 1) & 1];
        d.in[1] = I.src + ws;
        d.in[2] = I.src + hs * I.src_pitch;
        d.in[3] = I.src + hs * I.src_pitch + ws;
        d.in_pitch[1] = d.in_pitch[2] = d.in_pitch[3] = I.src_pitch;
        if (j == 1) {
            d.out[0] = I.dst;
            d.out_pitch[0] = I.dst_pitch;
        } else {
            d.out[0] = I.ll[(j - 2) & 1];
            d.out_pitch[0] = I.llp[(j - 2) & 1];
        }
        d.n_strips = I.n_strips[j - 1];
        d.seg_pairs = I.seg[j - 1];
        d.n_segs = I.n_segs[j - 1];
    }
    return d;
}

struct WarpSync {
    __device__ void operator()() const { __syncwarp(); }
};

// All levels from j_tail on in one warp, the band and its half-transformed
// copy in the warp's ring (row-major, odd pitch).
template <int NS>
__device__ void tail_item(const BatchImage &I, float *smem, int lane)
{
    const int j0 = I.j_tail;
    const int w0 = ceil_div_pow2(I.w, j0), h0 = ceil_div_pow2(I.h, j0);
    const int P = recur::band_pitch(w0);
    float *A = smem, *B = smem + P * h0;
    const Wavelet W = make_wavelet_dev(I.wavelet, I.inverse);
    const int levels = I.J - j0;
    const float *in = I.inverse ? I.src : (j0 == 0 ? I.src : I.ll[(j0 - 1) & 1]);
    const long long ip = I.inverse ? I.src_pitch : (j0 == 0 ? I.src_pitch : I.llp[(j0 - 1) & 1]);
    for (int y = 0; y < h0; ++y)
        for (int x = lane; x < w0; x += 32) A[y * P + x] = in[y * ip + x];
    __syncwarp();
    if (!I.inverse) {
        recur::band_forward<NS>(A, B, w0, h0, levels, I.dst, I.dst_pitch, W, lane, 32, WarpSync{});
    } else {
        recur::band_inverse<NS>(A, B, w0, h0, levels, W, lane, 32, WarpSync{});
        float *out = j0 == 0 ? I.dst : I.ll[(j0 - 1) & 1];
        const long long op = j0 == 0 ? I.dst_pitch : I.llp[(j0 - 1) & 1];
        for (int y = 0; y < h0; ++y)
            for (int x = lane; x < w0; x += 32) out[y * op + x] = A[y * P + x];
    }
    __syncwarp();
}

template <int NS, bool INV>
__device__ __forceinline__ bool level_item(const BatchImage &I, int level, int unit, float *ring, uint64_t *bars,
                                           uint32_t &tick, int lane, int *err)
{
    const LevelDesc D = level_desc(I, level);
    const Wavelet W = make_wavelet_dev(I.wavelet, INV);
    const int strip = unit % D.n_strips, seg = unit / D.n_strips;
    int unused = 0;
    return units::run_unit<NS, INV>(D, W, strip, seg, ring, bars, tick, lane, err, units::fast_ok<INV>(D), nullptr,
                                    unused);
}

__global__ void __launch_bounds__(kBatchWarps * 32)
batch_kernel(const BatchImage *__restrict__ imgs, const BatchItem *__restrict__ items, int n_items, int *ticket,
             int *done, int *err)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *ring = units::warp_ring(smem, warp);
    uint64_t *bars = units::warp_bars(smem, warp, kBatchWarps);
    units::init_bars(bars, lane);
    uint32_t tick = 0;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(ticket, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= n_items) break;
        const BatchItem it = items[t];
        const BatchImage &I = imgs[it.image];
        if (it.phase > 0) {
            // wait for the previous phase of this image (bounded)
            bool ok = true;
            if (lane == 0) {
                const int need = I.units[it.phase - 1];
                const int *cnt = done + it.image * kPhases + it.phase - 1;
                uint32_t spins = 0;
                while (ld_acquire(cnt) < need) {
                    __nanosleep(256);
                    if (++spins > (1u << 24)) {
                        atomicCAS(err, 0, kErrQueueTimeout);
                        ok = false;
                        break;
                    }
                }
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
            __syncwarp();
            fence_proxy_async_global();  // the TMA reads below see the other warps' stores
        }
        bool ok = true;
        if (it.level < 0) {
            if (I.wavelet == CDF97)
                tail_item<4>(I, ring, lane);
            else
                tail_item<2>(I, ring, lane);
            // the tail used the ring as plain shared memory: order those
            // accesses before the next item's TMA writes into it
            fence_proxy_async_smem();
        } else if (I.wavelet == CDF97) {
            ok = I.inverse ? level_item<4, true>(I, it.level, it.unit, ring, bars, tick, lane, err)
                           : level_item<4, false>(I, it.level, it.unit, ring, bars, tick, lane, err);
        } else {
            ok = I.inverse ? level_item<2, true>(I, it.level, it.unit, ring, bars, tick, lane, err)
                           : level_item<2, false>(I, it.level, it.unit, ring, bars, tick, lane, err);
        }
        if (!ok) break;
        // the warp's stores, then one release by lane 0 (cumulative over the
        // warp's writes ordered before it by the warp barrier)
        __syncwarp();
        if (lane == 0) {
            red_release_add(done + it.image * kPhases + it.phase, 1);
        }
    }
}

// ------------------------------------------------------------ host side

long long align_up_ll(long long v, long long a) { return (v + a - 1) / a * a; }

constexpr int kRingFloats = kStages * kStageFloats;

bool tail_fits(int w, int h, int side)
{
    return side > 0 && w <= side && h <= side && recur::band_floats(w, h) <= kRingFloats;
}

}  // namespace

}  // namespace dwt

using namespace dwt;

struct dwt_gpu_batch {
    int n = 0;
    std::vector<dwt_gpu_batch_image> images;
    dwt_gpu_batch_params params{};
    BatchImage *d_imgs = nullptr;
    BatchItem *d_items = nullptr;
    int *d_counters = nullptr;  // [0] ticket, [1..] done counters
    size_t counter_bytes = 0;
    int n_items = 0;
    void *arena = nullptr;
    cudaStream_t capture = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int grid = 0;
    std::vector<int> plain_copy;  // images with zero levels (copied as is)
};

namespace {

void release_plan(dwt_gpu_batch *b)
{
    Context &c = ctx();
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    if (b->d_imgs) c.pool.release(b->d_imgs, c.stream);
    if (b->d_items) c.pool.release(b->d_items, c.stream);
    if (b->d_counters) c.pool.release(b->d_counters, c.stream);
    if (b->arena) c.pool.release(b->arena, c.stream);
    b->d_imgs = nullptr;
    b->d_items = nullptr;
    b->d_counters = nullptr;
    b->arena = nullptr;
}

// Builds descriptors, items, scratch and the graph for the current params.
int build_plan(dwt_gpu_batch *b)
{
    Context &c = ctx();
    release_plan(b);
    const dwt_gpu_batch_params &P = b->params;
    std::vector<BatchImage> imgs(b->n);
    std::vector<std::vector<BatchItem>> by_phase(kPhases);
    std::vector<size_t> scratch_off(b->n);
    size_t arena_floats = 0;
    b->plain_copy.clear();
    for (int i = 0; i < b->n; ++i) {
        const size_t sf = plan_image(imgs[i], b->images[i], P, i, by_phase);
        if (imgs[i].J == 0) {
            b->plain_copy.push_back(i);
            continue;
        }
        scratch_off[i] = arena_floats;
        arena_floats += align_up_ll((long long)sf, 64);
    }
    // within a phase, the items of one (wavelet, direction) together: the
    // warps of an SM then mostly run one kernel variant at a time instead of
    // evicting each other's code from the instruction cache
    group_items_by_variant(by_phase, imgs);
    std::vector<BatchItem> items;
    for (auto &v : by_phase) items.insert(items.end(), v.begin(), v.end());
    b->n_items = int(items.size());

    cudaStream_t s = c.stream;
    b->arena = arena_floats ? c.pool.alloc(arena_floats * 4 + 256, s) : nullptr;
    b->d_imgs = static_cast<BatchImage *>(c.pool.alloc(sizeof(BatchImage) * std::max(1, b->n), s));
    b->d_items = static_cast<BatchItem *>(c.pool.alloc(sizeof(BatchItem) * std::max(1, b->n_items), s));
    b->counter_bytes = sizeof(int) * (1 + size_t(b->n) * kPhases);
    b->d_counters = static_cast<int *>(c.pool.alloc(b->counter_bytes, s));
    if ((arena_floats && !b->arena) || !b->d_imgs || !b->d_items || !b->d_counters) return DWT_GPU_ENOMEM;
    for (int i = 0; i < b->n; ++i)
        if (imgs[i].J > 0) set_image_scratch(imgs[i], static_cast<float *>(b->arena) + scratch_off[i]);
    if (cudaMemcpyAsync(b->d_imgs, imgs.data(), sizeof(BatchImage) * b->n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        (b->n_items && cudaMemcpyAsync(b->d_items, items.data(), sizeof(BatchItem) * b->n_items,
                                       cudaMemcpyHostToDevice, s) != cudaSuccess) ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return DWT_GPU_ECUDA;

    // the graph: zero the counters, copy zero-level images, run the kernel
    b->grid = std::max(1, std::min(c.sm_count * P.ctas_per_sm, (b->n_items + kBatchWarps - 1) / kBatchWarps));
    if (!b->capture && cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking) != cudaSuccess)
        return DWT_GPU_ECUDA;
    if (cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return DWT_GPU_ECUDA;
    cudaMemsetAsync(b->d_counters, 0, b->counter_bytes, b->capture);
    for (int i : b->plain_copy) {
        const dwt_gpu_batch_image &u = b->images[i];
        if (u.src != u.dst)
            cudaMemcpy2DAsync(u.dst, u.dst_pitch_bytes, u.src, u.src_pitch_bytes, size_t(u.w) * 4, u.h,
                              cudaMemcpyDeviceToDevice, b->capture);
    }
    if (b->n_items &&
        launch_batch_kernel(b->grid, b->d_imgs, b->d_items, b->n_items, b->d_counters, c.d_err, b->capture) !=
            cudaSuccess) {
        cudaGraph_t g;
        cudaStreamEndCapture(b->capture, &g);
        return DWT_GPU_ECUDA;
    }
    if (cudaStreamEndCapture(b->capture, &b->graph) != cudaSuccess) return DWT_GPU_ECUDA;
    if (cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess) return DWT_GPU_ECUDA;
    return DWT_GPU_OK;
}

}  // namespace

namespace dwt {

// Whether the items of a phase are grouped by kernel variant (default on;
// DWT_GPU_BATCH_GROUP_VARIANTS=0 keeps the image order).
static bool sort_phases_by_variant()
{
    static const bool on = [] {
        const char *v = getenv("DWT_GPU_BATCH_GROUP_VARIANTS");
        return !(v && v[0] == '0');
    }();
    return on;
}

void group_items_by_variant(std::vector<std::vector<BatchItem>> &by_phase, const std::vector<BatchImage> &imgs)
{
    if (!sort_phases_by_variant()) return;
    auto variant = [&](const BatchItem &it) { return imgs[it.image].wavelet * 2 + (imgs[it.image].inverse ? 1 : 0); };
    for (auto &v : by_phase)
        std::stable_sort(v.begin(), v.end(),
                         [&](const BatchItem &x, const BatchItem &y) { return variant(x) < variant(y); });
}


size_t plan_image(BatchImage &I, const dwt_gpu_batch_image &u, const dwt_gpu_batch_params &P, int i,
                  std::vector<std::vector<BatchItem>> &by_phase)
{
    memset(&I, 0, sizeof(I));
    const int lim = ceil_log2_int(u.decompose_one ? std::max(u.w, u.h) : std::min(u.w, u.h));
    const int J = (u.j_levels < 0 || u.j_levels > lim) ? lim : u.j_levels;
    I.src = u.src;
    I.src_pitch = u.src_pitch_bytes / 4;
    I.dst = u.dst;
    I.dst_pitch = u.dst_pitch_bytes / 4;
    I.w = u.w;
    I.h = u.h;
    I.J = J;
    I.wavelet = u.wavelet;
    I.inverse = u.inverse;
    if (J == 0) return 0;
    long long p0, p1;
    const size_t sf = dense_scratch_floats(u.w, u.h, J, &p0, &p1);
    I.llp[0] = p0;
    I.llp[1] = p1;
    // the first level whose band the tail item takes
    I.j_tail = J;
    for (int j = 0; j < J; ++j)
        if (tail_fits(ceil_div_pow2(u.w, j), ceil_div_pow2(u.h, j), P.tail_side)) {
            I.j_tail = j;
            break;
        }
    for (int j = 0; j < J; ++j) {
        const int w = ceil_div_pow2(u.w, j), h = ceil_div_pow2(u.h, j);
        const int npairs = (h == 1) ? 1 : (h + 1) / 2;
        I.n_strips[j] = ceil_div(w, kStripOut);
        I.seg[j] = std::max(1, std::min(P.seg_pairs, npairs));
        I.n_segs[j] = ceil_div(npairs, I.seg[j]);
    }
    int phase = 0;
    auto level_units = [&](int jidx) { return I.n_strips[jidx] * I.n_segs[jidx]; };
    if (!u.inverse) {
        for (int j = 0; j < I.j_tail; ++j, ++phase) {
            I.units[phase] = level_units(j);
            for (int k = 0; k < I.units[phase]; ++k) by_phase[phase].push_back({i, phase, j, k});
        }
        if (I.j_tail < J) {
            I.units[phase] = 1;
            by_phase[phase].push_back({i, phase, -1, 0});
        }
    } else {
        int jtop = J;
        if (I.j_tail < J) {
            I.units[phase] = 1;
            by_phase[phase].push_back({i, phase, -1, 0});
            ++phase;
            jtop = I.j_tail;
        }
        for (int j = jtop; j >= 1; --j, ++phase) {
            I.units[phase] = level_units(j - 1);
            for (int k = 0; k < I.units[phase]; ++k) by_phase[phase].push_back({i, phase, j, k});
        }
    }
    return sf;
}

void set_image_scratch(BatchImage &I, float *scratch)
{
    long long p0, p1;
    dense_scratch_floats(I.w, I.h, I.J, &p0, &p1);
    I.ll[0] = scratch;
    I.ll[1] = scratch + (I.J >= 2 ? size_t(p0) * ((I.h + 1) / 2) + 64 : 0);
}

int batch_smem_bytes() { return kBatchWarps * (kStages * kStageFloats * 4 + kStages * 8); }

cudaError_t launch_batch_kernel(int grid, const BatchImage *imgs, const BatchItem *items, int n_items,
                                int *counters, int *err, cudaStream_t s)
{
    // once per process, safe from several host threads
    static const cudaError_t configured =
        cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, batch_smem_bytes());
    if (configured != cudaSuccess) return configured;
    batch_kernel<<<grid, kBatchWarps * 32, batch_smem_bytes(), s>>>(imgs, items, n_items, counters, counters + 1, err);
    return cudaGetLastError();
}

}  // namespace dwt

namespace {

// --------------------------------------------------------------- autotuner

std::string signature(const dwt_gpu_batch *b)
{
    // count, pixel total, mix of wavelets and directions, log2 size histogram
    long long px = 0;
    int hist[24] = {0}, n97 = 0, ninv = 0;
    for (const auto &u : b->images) {
        px += (long long)u.w * u.h;
        const long long a = (long long)u.w * u.h;
        int lg = 0;
        while ((1LL << (lg + 1)) <= a && lg < 23) ++lg;
        hist[lg]++;
        n97 += u.wavelet == CDF97;
        ninv += u.inverse != 0;
    }
    std::ostringstream os;
    os << b->n << ":" << px << ":" << n97 << ":" << ninv;
    for (int k = 0; k < 24; ++k)
        if (hist[k]) os << ":" << k << "x" << hist[k];
    return os.str();
}

std::string cache_path()
{
    const char *p = getenv("DWT_GPU_TUNE_CACHE");
    if (p && *p) return p;
    const char *home = getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/libdwt_gb300_batch_tune.txt";
}

std::mutex g_tune_mu;

bool cache_lookup(const std::string &sig, dwt_gpu_batch_params *out)
{
    std::lock_guard<std::mutex> g(g_tune_mu);
    std::ifstream f(cache_path());
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        std::string s;
        dwt_gpu_batch_params p{};
        if (is >> s >> p.seg_pairs >> p.tail_side >> p.ctas_per_sm && s == sig) {
            *out = p;
            return true;
        }
    }
    return false;
}

void cache_store(const std::string &sig, const dwt_gpu_batch_params &p)
{
    std::lock_guard<std::mutex> g(g_tune_mu);
    const std::string path = cache_path();
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos) {
        const std::string dir = path.substr(0, slash);
        std::string cmd_dir = dir;  // create the directory if needed
        if (!cmd_dir.empty()) {
            std::string mk = "mkdir -p '" + cmd_dir + "' 2>/dev/null";
            if (system(mk.c_str()) != 0) { /* the write below reports nothing either */ }
        }
    }
    std::ofstream f(path, std::ios::app);
    f << sig << " " << p.seg_pairs << " " << p.tail_side << " " << p.ctas_per_sm << "\n";
}

float time_plan(dwt_gpu_batch *b, int reps)
{
    Context &c = ctx();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaGraphLaunch(b->exec, c.stream);
    cudaEventRecord(e0, c.stream);
    for (int r = 0; r < reps; ++r) cudaGraphLaunch(b->exec, c.stream);
    cudaEventRecord(e1, c.stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms / reps;
}

int autotune(dwt_gpu_batch *b)
{
    const std::string sig = signature(b);
    dwt_gpu_batch_params best{};
    if (cache_lookup(sig, &best)) {
        b->params = best;
        return build_plan(b);
    }
    const int segs[] = {8, 16, 32, 64};
    const int tails[] = {0, 16, 32};
    const int ctas[] = {4, 6};
    float best_ms = 1e30f;
    for (int sp : segs)
        for (int ts : tails)
            for (int cp : ctas) {
                b->params = dwt_gpu_batch_params{sp, ts, cp};
                if (build_plan(b) != DWT_GPU_OK) continue;
                const float ms = time_plan(b, 3);
                if (ms < best_ms) {
                    best_ms = ms;
                    best = b->params;
                }
            }
    if (best_ms >= 1e30f) return DWT_GPU_ECUDA;
    cache_store(sig, best);
    b->params = best;
    return build_plan(b);
}

}  // namespace

extern "C" {

int dwt_gpu_batch_create(dwt_gpu_batch **out, int n, const dwt_gpu_batch_image *images,
                         const dwt_gpu_batch_params *params)
{
    if (!out || n < 0 || (n > 0 && !images)) return set_error(DWT_GPU_EINVAL);
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        const dwt_gpu_batch_image &u = images[i];
        if (u.w <= 0 || u.h <= 0 || !u.src || !u.dst || (u.src_pitch_bytes % 16) != 0 ||
            (reinterpret_cast<uintptr_t>(u.src) & 15) != 0 || (u.dst_pitch_bytes % 4) != 0 ||
            u.src_pitch_bytes < 4LL * u.w || u.dst_pitch_bytes < 4LL * u.w ||
            (u.wavelet != CDF97 && u.wavelet != CDF53)) {
            log_error("dwt_gpu_batch_create: image %d has invalid arguments\n", i);
            return set_error(DWT_GPU_EINVAL);
        }
    }
    dwt_gpu_batch *b = new dwt_gpu_batch();
    b->n = n;
    b->images.assign(images, images + n);
    int rc;
    if (params) {
        b->params = *params;
        if (b->params.seg_pairs <= 0) b->params.seg_pairs = 16;
        if (b->params.ctas_per_sm <= 0) b->params.ctas_per_sm = 4;
        rc = build_plan(b);
    } else {
        rc = autotune(b);
    }
    if (rc != DWT_GPU_OK) {
        release_plan(b);
        delete b;
        return set_error(rc);
    }
    *out = b;
    return set_error(DWT_GPU_OK);
}

int dwt_gpu_batch_run(dwt_gpu_batch *b, void *stream)
{
    if (!b) return set_error(DWT_GPU_EINVAL);
    if (cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream)) != cudaSuccess) return set_error(DWT_GPU_ECUDA);
    return set_error(DWT_GPU_OK);
}

int dwt_gpu_batch_params_get(const dwt_gpu_batch *b, dwt_gpu_batch_params *p)
{
    if (!b || !p) return set_error(DWT_GPU_EINVAL);
    *p = b->params;
    return DWT_GPU_OK;
}

int dwt_gpu_batch_items(const dwt_gpu_batch *b) { return b ? b->n_items : -1; }

void dwt_gpu_batch_destroy(dwt_gpu_batch *b)
{
    if (!b) return;
    cudaStreamSynchronize(ctx().stream);
    release_plan(b);
    if (b->capture) cudaStreamDestroy(b->capture);
    delete b;
}

}  // extern "C"
