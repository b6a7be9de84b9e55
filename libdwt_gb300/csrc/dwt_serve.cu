// Serving loop: continuous batching of 2D transform requests.
//
// Clients submit requests (device frames in, device frame or a pooled buffer
// out, size, wavelet, direction, levels) at any time.  A dispatcher thread
//   - admits pending requests in arrival order while their device memory
//     (pooled output buffer if the client gave none, plus the inter-level
//     scratch) fits the memory budget and an in-flight slot is free;
//   - turns everything admitted since the last launch into one micro-batch
//     on the next of several streams, so micro-batches overlap on the device
//     and requests that arrive while others run join the next one: the small
//     requests become descriptors and work items of the batched persistent
//     kernel, the large ones (kDenseMinPixels and up, most of the pixels of
//     a mixed stream) run the per-level pipeline of the plain drop-in, which
//     is at its best on large images;
//   - polls the micro-batches' completion events, returns their buffers to
//     the server's arena and stamps each request's completion time.
// Device memory: every request's output (when the client gave none) and
// inter-level scratch come from the server's own arena (dwt_arena.h), slabs
// reserved at set-up by dwt_gpu_server_reserve, so that no cudaMalloc or
// cudaFree runs on the dispatcher while requests are served; each flight
// keeps its descriptor buffers (device and pinned host) for its lifetime.
// dwt_gpu_server_reserve also runs one small and one large request of every
// wavelet and direction, so the kernels are loaded and configured before the
// first client request.
// Latency is arrival (submit) to completion as seen by the dispatcher.
// dwt_gpu_server_replay drives a recorded arrival trace in real time (the
// benchmark's Poisson stream) from the calling thread.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/libdwt.h"
#include "dwt_arena.h"
#include "dwt_batch.cuh"
#include "dwt_capi_internal.h"

namespace {

using dwt::BatchImage;
using dwt::BatchItem;

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Req {
    long long id;
    dwt_gpu_request r;
    double t_submit = 0, t_admit = 0, t_done = 0;
    float *pooled = nullptr;  // pooled output when the client gave no dst
    void *scratch = nullptr;
    size_t bytes = 0;  // budget charge
    int status = 0;
};

struct Flight {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    std::vector<Req> reqs;
    void *d_desc = nullptr;  // images + items + counters (kept, grown when too small)
    size_t d_cap = 0;
    void *h_desc = nullptr;  // pinned staging of the descriptors (kept, grown likewise)
    size_t h_cap = 0;
    bool busy = false;
};

// Descriptor capacity each flight starts with (device and pinned host): a
// micro-batch of small requests holds at most about kFlightPixels / 4096 work
// items, far below this.
constexpr size_t kDescBytes = size_t(8) << 20;

}  // namespace

struct dwt_gpu_server {
    size_t budget = 0;
    std::atomic<size_t> used{0};
    size_t peak = 0;
    dwt_gpu_batch_params params{};
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Req> pending;
    std::vector<dwt_gpu_completion> completed;
    std::vector<Flight> flights;
    int next_flight = 0;
    long long next_id = 1;
    long long submitted = 0, finished = 0, launches = 0, admitted = 0;
    std::atomic<bool> stop{false};
    std::thread dispatcher;
    int device = 0;
    dwt::Arena arena;
    std::atomic<long long> desc_allocs{0};     // descriptor buffers grown after set-up
    std::atomic<long long> max_loop_ns{0};     // longest dispatcher iteration
};

namespace {

size_t request_bytes(const dwt_gpu_request &r, int J)
{
    long long p0, p1;
    const size_t sf = dwt::dense_scratch_floats(r.w, r.h, J, &p0, &p1);
    return sf * 4 + 256 + (r.dst ? 0 : size_t(r.w) * r.h * 4 + 256);
}

// Requests of at least this many pixels take the per-level pipeline.
constexpr long long kDenseMinPixels = 1LL << 21;
// A micro-batch takes requests until it holds this many pixels (about 0.3 ms
// of GPU work): long micro-batches would leave the other streams idle while
// the last of their work drains, and hold every request to the slowest.
constexpr long long kFlightPixels = 1LL << 27;

bool dense_request(const dwt_gpu_request &r) { return (long long)r.w * r.h >= kDenseMinPixels; }

int levels_of(const dwt_gpu_request &r)
{
    const int lim = dwt::ceil_log2_int(r.decompose_one ? std::max(r.w, r.h) : std::min(r.w, r.h));
    return (r.j_levels < 0 || r.j_levels > lim) ? lim : r.j_levels;
}

// Launches one micro-batch on flight f (its reqs already admitted).
void launch_flight(dwt_gpu_server *S, Flight &f)
{
    dwt::Context &c = dwt::ctx();
    std::vector<BatchImage> imgs;
    imgs.reserve(f.reqs.size());
    std::vector<std::vector<BatchItem>> by_phase(dwt::kPhases);
    std::vector<int> copies, dense;
    for (size_t i = 0; i < f.reqs.size(); ++i) {
        Req &q = f.reqs[i];
        if (dense_request(q.r) && levels_of(q.r) > 0) {
            dense.push_back(int(i));
            continue;
        }
        dwt_gpu_batch_image u{q.r.src, q.r.src_pitch_bytes,
                              q.r.dst ? q.r.dst : q.pooled,
                              q.r.dst ? q.r.dst_pitch_bytes : (long long)q.r.w * 4,
                              q.r.w, q.r.h, q.r.j_levels, q.r.decompose_one, q.r.wavelet, q.r.inverse};
        imgs.emplace_back();
        dwt::plan_image(imgs.back(), u, S->params, int(imgs.size() - 1), by_phase);
        if (imgs.back().J == 0)
            copies.push_back(int(i));
        else
            dwt::set_image_scratch(imgs.back(), static_cast<float *>(q.scratch));
    }
    dwt::group_items_by_variant(by_phase, imgs);
    size_t n_items = 0;
    for (auto &v : by_phase) n_items += v.size();
    const size_t img_b = sizeof(BatchImage) * imgs.size();
    const size_t item_b = sizeof(BatchItem) * n_items;
    const size_t cnt_b = sizeof(int) * (1 + imgs.size() * dwt::kPhases);
    const size_t off_items = (img_b + 255) & ~size_t(255);
    const size_t off_cnt = (off_items + item_b + 255) & ~size_t(255);
    const size_t total = off_cnt + cnt_b;
    if (f.d_cap < total) {
        // only a micro-batch beyond kDescBytes gets here; the flight's stream
        // is idle (the flight was free), so the old buffers can go at once
        S->desc_allocs++;
        if (f.d_desc) cudaFree(f.d_desc);
        f.d_cap = std::max(total, 2 * f.d_cap);
        if (cudaMalloc(&f.d_desc, f.d_cap) != cudaSuccess) {
            cudaGetLastError();
            f.d_desc = nullptr;
            f.d_cap = 0;
        }
    }
    if (f.h_cap < off_cnt) {
        S->desc_allocs++;
        if (f.h_desc) cudaFreeHost(f.h_desc);
        f.h_cap = std::max(off_cnt, 2 * f.h_cap);
        if (cudaHostAlloc(&f.h_desc, f.h_cap, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            f.h_desc = nullptr;
            f.h_cap = 0;
        }
    }
    if (!f.d_desc || !f.h_desc) {
        for (Req &q : f.reqs) q.status = DWT_GPU_ENOMEM;
        cudaEventRecord(f.done, f.stream);
        f.busy = true;
        return;
    }
    char *h = static_cast<char *>(f.h_desc);
    memcpy(h, imgs.data(), img_b);
    char *p = h + off_items;
    for (auto &v : by_phase) {
        memcpy(p, v.data(), sizeof(BatchItem) * v.size());
        p += sizeof(BatchItem) * v.size();
    }
    char *d = static_cast<char *>(f.d_desc);
    cudaMemcpyAsync(d, h, off_cnt, cudaMemcpyHostToDevice, f.stream);
    cudaMemsetAsync(d + off_cnt, 0, cnt_b, f.stream);
    for (int i : copies) {
        const Req &q = f.reqs[i];
        float *dst = q.r.dst ? q.r.dst : q.pooled;
        const long long dp = q.r.dst ? q.r.dst_pitch_bytes : (long long)q.r.w * 4;
        cudaMemcpy2DAsync(dst, dp, q.r.src, q.r.src_pitch_bytes, size_t(q.r.w) * 4, q.r.h,
                          cudaMemcpyDeviceToDevice, f.stream);
    }
    if (n_items) {
        const int grid = std::max(1, std::min(c.sm_count * S->params.ctas_per_sm, int((n_items + 3) / 4)));
        dwt::launch_batch_kernel(grid, reinterpret_cast<BatchImage *>(d), reinterpret_cast<BatchItem *>(d + off_items),
                                 int(n_items), reinterpret_cast<int *>(d + off_cnt), c.d_err, f.stream);
    }
    for (int i : dense) {
        Req &q = f.reqs[i];
        float *dst = q.r.dst ? q.r.dst : q.pooled;
        const long long dp = (q.r.dst ? q.r.dst_pitch_bytes : (long long)q.r.w * 4) / 4;
        const int J = levels_of(q.r);
        const cudaError_t e =
            q.r.inverse ? dwt::dense_inverse(q.r.src, q.r.src_pitch_bytes / 4, dst, dp, q.r.w, q.r.h, J, q.r.wavelet,
                                             static_cast<float *>(q.scratch), f.stream, c.d_err, 0)
                        : dwt::dense_forward(q.r.src, q.r.src_pitch_bytes / 4, dst, dp, q.r.w, q.r.h, J, q.r.wavelet,
                                             static_cast<float *>(q.scratch), f.stream, c.d_err, 0);
        if (e != cudaSuccess) q.status = DWT_GPU_ECUDA;
    }
    cudaEventRecord(f.done, f.stream);
    f.busy = true;
}

void dispatcher_loop(dwt_gpu_server *S)
{
    cudaSetDevice(S->device);
    std::vector<Req> admitted;
    while (!S->stop.load()) {
        bool did = false;
        const double t_loop = now_s();
        // 1. completions
        for (Flight &f : S->flights) {
            if (!f.busy || cudaEventQuery(f.done) != cudaSuccess) continue;
            const double t = now_s();
            std::vector<dwt_gpu_completion> done;
            for (Req &q : f.reqs) {
                S->arena.free(q.pooled);
                S->arena.free(q.scratch);
                S->used -= q.bytes;
                done.push_back({q.id, q.r.tag, q.status, q.t_submit, q.t_admit, t});
            }
            f.reqs.clear();
            f.busy = false;
            {
                std::lock_guard<std::mutex> g(S->mu);
                S->completed.insert(S->completed.end(), done.begin(), done.end());
                S->finished += (long long)done.size();
            }
            S->cv.notify_all();
            did = true;
        }
        // 2. admission, in arrival order, while memory and a free flight allow
        Flight *free_f = nullptr;
        for (int k = 0; k < int(S->flights.size()); ++k) {
            Flight &f = S->flights[(S->next_flight + k) % S->flights.size()];
            if (!f.busy) {
                free_f = &f;
                S->next_flight = int((&f - S->flights.data() + 1) % S->flights.size());
                break;
            }
        }
        if (free_f) {
            std::unique_lock<std::mutex> g(S->mu);
            long long flight_px = 0;
            while (!S->pending.empty() && flight_px < kFlightPixels) {
                Req &q = S->pending.front();
                const int J = levels_of(q.r);
                const size_t need = request_bytes(q.r, J);
                if (S->used + need > S->budget) break;
                long long p0, p1;
                const size_t sf = dwt::dense_scratch_floats(q.r.w, q.r.h, J, &p0, &p1);
                void *scratch = sf ? S->arena.alloc(sf * 4 + 256) : nullptr;
                void *pooled = q.r.dst ? nullptr : S->arena.alloc(size_t(q.r.w) * q.r.h * 4 + 256);
                if ((sf && !scratch) || (!q.r.dst && !pooled)) {
                    S->arena.free(scratch);
                    S->arena.free(pooled);
                    // the arena is full (or fragmented) at its cap: wait for
                    // completions to free memory; with nothing in flight its
                    // slabs are too small for this request, so they are
                    // replaced by one that holds it (a rare, synchronising path)
                    if (S->used.load() == 0 && S->arena.release_if_idle()) continue;
                    break;
                }
                q.scratch = scratch;
                q.pooled = static_cast<float *>(pooled);
                flight_px += (long long)q.r.w * q.r.h;
                q.bytes = need;
                S->used += need;
                S->peak = std::max(S->peak, S->used.load());
                admitted.push_back(q);
                S->pending.pop_front();
            }
            g.unlock();
            if (!admitted.empty()) {
                const double t = now_s();
                for (Req &q : admitted) q.t_admit = t;
                free_f->reqs.swap(admitted);
                admitted.clear();
                S->admitted += (long long)free_f->reqs.size();
                S->launches++;
                launch_flight(S, *free_f);
                did = true;
            }
        }
        const double t_end = now_s();
        const long long ns = (long long)((t_end - t_loop) * 1e9);
        if (ns > S->max_loop_ns.load()) S->max_loop_ns = ns;
        if (!did) std::this_thread::sleep_for(std::chrono::microseconds(5));
    }
}

}  // namespace

extern "C" {

int dwt_gpu_server_create(dwt_gpu_server **out, long long budget_bytes, int n_streams,
                          const dwt_gpu_batch_params *params)
{
    if (!out || budget_bytes <= 0) return dwt::set_error(DWT_GPU_EINVAL);
    dwt::Context &c = dwt::ctx();
    dwt_gpu_server *S = new dwt_gpu_server();
    S->device = c.device;
    S->budget = size_t(budget_bytes);
    S->params = params ? *params : dwt_gpu_batch_params{32, 32, 4};
    if (S->params.seg_pairs <= 0) S->params.seg_pairs = 32;
    if (S->params.ctas_per_sm <= 0) S->params.ctas_per_sm = 4;
    S->arena.set_cap(S->budget);
    S->flights.resize(std::max(1, n_streams));
    for (Flight &f : S->flights) {
        cudaStreamCreateWithFlags(&f.stream, cudaStreamNonBlocking);
        cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming);
        if (cudaMalloc(&f.d_desc, kDescBytes) == cudaSuccess) f.d_cap = kDescBytes;
        else f.d_desc = nullptr;
        if (cudaHostAlloc(&f.h_desc, kDescBytes, cudaHostAllocDefault) == cudaSuccess) f.h_cap = kDescBytes;
        else f.h_desc = nullptr;
        cudaGetLastError();
    }
    S->dispatcher = std::thread(dispatcher_loop, S);
    *out = S;
    return dwt::set_error(DWT_GPU_OK);
}

int dwt_gpu_server_submit(dwt_gpu_server *S, const dwt_gpu_request *r, long long *id)
{
    if (!S || !r || r->w <= 0 || r->h <= 0 || !r->src || (r->src_pitch_bytes % 16) != 0 ||
        (reinterpret_cast<uintptr_t>(r->src) & 15) != 0 || r->src_pitch_bytes < 4LL * r->w ||
        (r->dst && ((r->dst_pitch_bytes % 4) != 0 || r->dst_pitch_bytes < 4LL * r->w)) ||
        (r->wavelet != DWT_GPU_CDF97 && r->wavelet != DWT_GPU_CDF53))
        return dwt::set_error(DWT_GPU_EINVAL);
    if (request_bytes(*r, levels_of(*r)) > S->budget) return dwt::set_error(DWT_GPU_EBUSY);
    Req q;
    q.r = *r;
    q.t_submit = now_s();
    {
        std::lock_guard<std::mutex> g(S->mu);
        q.id = S->next_id++;
        S->pending.push_back(q);
        S->submitted++;
    }
    if (id) *id = q.id;
    return DWT_GPU_OK;
}

int dwt_gpu_server_poll(dwt_gpu_server *S, dwt_gpu_completion *out, int max, int *n)
{
    if (!S || !n || (max > 0 && !out)) return dwt::set_error(DWT_GPU_EINVAL);
    std::lock_guard<std::mutex> g(S->mu);
    const int k = std::min<int>(max, int(S->completed.size()));
    for (int i = 0; i < k; ++i) out[i] = S->completed[i];
    S->completed.erase(S->completed.begin(), S->completed.begin() + k);
    *n = k;
    return DWT_GPU_OK;
}

int dwt_gpu_server_drain(dwt_gpu_server *S, double timeout_s)
{
    if (!S) return dwt::set_error(DWT_GPU_EINVAL);
    std::unique_lock<std::mutex> g(S->mu);
    const bool ok = S->cv.wait_for(g, std::chrono::duration<double>(timeout_s),
                                   [S] { return S->finished == S->submitted; });
    return ok ? DWT_GPU_OK : dwt::set_error(DWT_GPU_EBUSY);
}

int dwt_gpu_server_stats(dwt_gpu_server *S, dwt_gpu_server_stats_t *st)
{
    if (!S || !st) return dwt::set_error(DWT_GPU_EINVAL);
    std::lock_guard<std::mutex> g(S->mu);
    st->submitted = S->submitted;
    st->completed = S->finished;
    st->launches = S->launches;
    st->pending = (long long)S->pending.size();
    st->bytes_in_use = (long long)S->used.load();
    st->peak_bytes = (long long)S->peak;
    st->budget_bytes = (long long)S->budget;
    const dwt::Arena::Stats a = S->arena.stats();
    st->arena_bytes = (long long)a.reserved;
    st->device_allocs = a.device_allocs + S->desc_allocs.load();
    st->max_dispatch_ns = S->max_loop_ns.load();
    return DWT_GPU_OK;
}

int dwt_gpu_server_reserve(dwt_gpu_server *S, long long bytes)
{
    if (!S || bytes < 0) return dwt::set_error(DWT_GPU_EINVAL);
    if (!S->arena.reserve(size_t(bytes))) return dwt::set_error(DWT_GPU_ENOMEM);
    // warm-up: one request of each path (batched kernel, small and odd; the
    // per-level pipeline with the coarse kernel) per wavelet and direction,
    // out of a zeroed source, so that every kernel the server launches is
    // loaded and configured now; their completions are dropped
    const int kw = 2048, kh = 1024;
    float *src = nullptr;
    if (cudaMalloc(&src, size_t(kw) * kh * 4) != cudaSuccess) {
        cudaGetLastError();
        return dwt::set_error(DWT_GPU_ENOMEM);
    }
    cudaMemset(src, 0, size_t(kw) * kh * 4);
    cudaDeviceSynchronize();
    std::vector<long long> ids;
    const int sizes[3][2] = {{64, 64}, {333, 97}, {kw, kh}};
    for (int wav : {DWT_GPU_CDF97, DWT_GPU_CDF53})
        for (int inv = 0; inv < 2; ++inv)
            for (const auto &sz : sizes) {
                dwt_gpu_request r{};
                r.src = src;
                r.src_pitch_bytes = (long long)kw * 4;
                r.dst = nullptr;
                r.w = sz[0];
                r.h = sz[1];
                r.j_levels = 6;
                r.wavelet = wav;
                r.inverse = inv;
                long long id = 0;
                if (dwt_gpu_server_submit(S, &r, &id) == DWT_GPU_OK) ids.push_back(id);
            }
    const int rc = dwt_gpu_server_drain(S, 120.0);
    cudaFree(src);
    {
        // the warm-up requests are not the clients': drop their completions
        // and start the counters afresh
        std::lock_guard<std::mutex> g(S->mu);
        S->completed.erase(std::remove_if(S->completed.begin(), S->completed.end(),
                                          [&](const dwt_gpu_completion &c) {
                                              return std::find(ids.begin(), ids.end(), c.id) != ids.end();
                                          }),
                           S->completed.end());
        if (rc == DWT_GPU_OK) {
            S->submitted -= (long long)ids.size();
            S->finished -= (long long)ids.size();
            S->admitted -= (long long)ids.size();
            S->launches = 0;
            S->peak = S->used.load();
        }
    }
    S->max_loop_ns = 0;
    return dwt::set_error(rc);
}

int dwt_gpu_server_replay(dwt_gpu_server *S, int n, const double *arrival_s, const dwt_gpu_request *reqs,
                          double *latency_s, double timeout_s)
{
    if (!S || n < 0 || (n > 0 && (!arrival_s || !reqs || !latency_s))) return dwt::set_error(DWT_GPU_EINVAL);
    std::vector<long long> ids(n, 0);
    S->max_loop_ns = 0;
    const double t0 = now_s();
    for (int i = 0; i < n; ++i) {
        const double due = t0 + arrival_s[i];
        while (now_s() < due) {
        }
        long long id = 0;
        if (dwt_gpu_server_submit(S, &reqs[i], &id) != DWT_GPU_OK) return dwt::set_error(DWT_GPU_EINVAL);
        ids[i] = id;
    }
    if (dwt_gpu_server_drain(S, timeout_s) != DWT_GPU_OK) return dwt::set_error(DWT_GPU_EBUSY);
    // collect the latencies by id
    std::vector<dwt_gpu_completion> all;
    {
        std::lock_guard<std::mutex> g(S->mu);
        all.swap(S->completed);
    }
    const long long first = ids.empty() ? 0 : ids[0];
    for (const auto &c : all) {
        const long long k = c.id - first;
        if (k >= 0 && k < n) latency_s[k] = c.t_complete - c.t_submit;
    }
    return DWT_GPU_OK;
}

void dwt_gpu_server_destroy(dwt_gpu_server *S)
{
    if (!S) return;
    dwt_gpu_server_drain(S, 60.0);
    S->stop = true;
    if (S->dispatcher.joinable()) S->dispatcher.join();
    for (Flight &f : S->flights) {
        cudaStreamSynchronize(f.stream);
        if (f.d_desc) cudaFree(f.d_desc);
        if (f.h_desc) cudaFreeHost(f.h_desc);
        cudaEventDestroy(f.done);
        cudaStreamDestroy(f.stream);
    }
    delete S;
}

}  // extern "C"
