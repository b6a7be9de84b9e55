// Stream-ordered caching device allocator.
//
// Blocks are cudaMalloc'ed once and kept on a free list after release.  A
// released block remembers the stream it was last used on and an event
// recorded there; handing it out on another stream makes that stream wait
// on the event first, so reuse never races with work still in flight.
// Sizes are rounded to buckets (powers of two below 4 MiB, 2 MiB multiples
// above) and a request is served by the smallest cached block that is at
// most twice its size.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <map>
#include <mutex>
#include <unordered_map>
#include <vector>

namespace dwt {

class Pool {
public:
    struct Stats {
        size_t in_use = 0, cached = 0, peak = 0, allocs = 0, hits = 0;
    };

    ~Pool() { release_all(); }

    static size_t bucket(size_t bytes)
    {
        if (bytes == 0) bytes = 1;
        if (bytes >= (size_t(4) << 20)) return (bytes + (size_t(2) << 20) - 1) & ~((size_t(2) << 20) - 1);
        size_t b = 4096;
        while (b < bytes) b <<= 1;
        return b;
    }

    // Returns nullptr on failure (out of memory after trimming the cache).
    void *alloc(size_t bytes, cudaStream_t stream)
    {
        const size_t want = bucket(bytes);
        std::lock_guard<std::mutex> g(mu_);
        auto it = free_.lower_bound(want);
        if (it != free_.end() && it->first <= 2 * want) {
            Block blk = it->second;
            free_.erase(it);
            if (blk.stream != stream && blk.event) cudaStreamWaitEvent(stream, blk.event, 0);
            blk.stream = stream;
            live_[blk.ptr] = blk;
            stats_.cached -= blk.size;
            stats_.in_use += blk.size;
            stats_.hits++;
            bump_peak();
            return blk.ptr;
        }
        void *p = nullptr;
        if (cudaMalloc(&p, want) != cudaSuccess) {
            cudaGetLastError();
            trim_locked();
            if (cudaMalloc(&p, want) != cudaSuccess) {
                cudaGetLastError();
                return nullptr;
            }
        }
        Block blk{p, want, stream, nullptr};
        live_[p] = blk;
        stats_.in_use += want;
        stats_.allocs++;
        bump_peak();
        return p;
    }

    void release(void *p, cudaStream_t stream)
    {
        if (!p) return;
        std::lock_guard<std::mutex> g(mu_);
        auto it = live_.find(p);
        if (it == live_.end()) return;
        Block blk = it->second;
        live_.erase(it);
        if (!blk.event) cudaEventCreateWithFlags(&blk.event, cudaEventDisableTiming);
        cudaEventRecord(blk.event, stream);
        blk.stream = stream;
        stats_.in_use -= blk.size;
        stats_.cached += blk.size;
        free_.emplace(blk.size, blk);
    }

    void trim()
    {
        std::lock_guard<std::mutex> g(mu_);
        trim_locked();
    }

    void release_all()
    {
        std::lock_guard<std::mutex> g(mu_);
        trim_locked();
        for (auto &kv : live_) {
            cudaFree(kv.second.ptr);
            if (kv.second.event) cudaEventDestroy(kv.second.event);
        }
        live_.clear();
        stats_.in_use = 0;
    }

    Stats stats()
    {
        std::lock_guard<std::mutex> g(mu_);
        return stats_;
    }

private:
    struct Block {
        void *ptr;
        size_t size;
        cudaStream_t stream;
        cudaEvent_t event;
    };

    void trim_locked()
    {
        for (auto &kv : free_) {
            if (kv.second.event) {
                cudaEventSynchronize(kv.second.event);
                cudaEventDestroy(kv.second.event);
            }
            cudaFree(kv.second.ptr);
        }
        free_.clear();
        stats_.cached = 0;
    }

    void bump_peak()
    {
        if (stats_.in_use > stats_.peak) stats_.peak = stats_.in_use;
    }

    std::mutex mu_;
    std::multimap<size_t, Block> free_;
    std::unordered_map<void *, Block> live_;
    Stats stats_;
};

}  // namespace dwt
