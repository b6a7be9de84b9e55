// Device memory arena of the serving loop.
//
// The server reserves its device memory up front, in a few large slabs
// (cudaMalloc'ed once, at set-up), and carves every request's buffers out of
// them: best fit by size, split on allocation, merged with free neighbours on
// release.  No cudaMalloc or cudaFree runs on the dispatcher thread while
// requests are served (both may synchronise the device and take milliseconds,
// which every request arriving meanwhile would wait for); only a request that
// fits nowhere grows the arena by one more slab, up to the cap.
//
// Buffers are released only after the GPU work that used them completed
// (the dispatcher has seen the micro-batch's completion event), so a range is
// reusable at once, on any stream, without events.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <map>
#include <mutex>
#include <unordered_map>
#include <vector>

namespace dwt {

// Where slabs come from: device memory (the host-memory backing of the unit
// test exercises the same bookkeeping on a machine without a GPU).
struct CudaBacking {
    static void *alloc(size_t bytes)
    {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return p;
    }
    static void free(void *p) { cudaFree(p); }
};

template <class Backing = CudaBacking>
class ArenaT {
public:
    static constexpr size_t kAlign = 256;
    static constexpr size_t kGrowBytes = size_t(1) << 30;  // one slab when a request fits nowhere

    ~ArenaT() { release(); }

    // Upper bound of the reserved bytes (slabs are never larger in total).
    void set_cap(size_t cap)
    {
        std::lock_guard<std::mutex> g(mu_);
        cap_ = cap;
    }

    // Adds slabs until at least `bytes` are reserved (slabs of at most 8 GiB,
    // so that a fragmented device can still serve them).  False if cudaMalloc
    // failed; what was reserved stays.
    bool reserve(size_t bytes)
    {
        std::lock_guard<std::mutex> g(mu_);
        bytes = std::min(bytes, cap_);
        while (reserved_ < bytes) {
            const size_t want = round_up(std::min(bytes - reserved_, size_t(8) << 30), size_t(2) << 20);
            if (!grow_locked(want)) return false;
        }
        return true;
    }

    // A buffer of `bytes` (256-byte aligned), or nullptr when no free range
    // fits and the cap forbids another slab.
    void *alloc(size_t bytes)
    {
        const size_t n = round_up(bytes ? bytes : 1, kAlign);
        std::lock_guard<std::mutex> g(mu_);
        void *p = take_locked(n);
        if (!p && reserved_ < cap_) {
            const size_t want = std::min(std::max(kGrowBytes, round_up(n, size_t(2) << 20)), cap_ - reserved_);
            if (want >= n && grow_locked(want)) p = take_locked(n);
        }
        if (p) {
            in_use_ += live_[static_cast<char *>(p)].size;
            if (in_use_ > peak_) peak_ = in_use_;
        }
        return p;
    }

    void free(void *ptr)
    {
        if (!ptr) return;
        std::lock_guard<std::mutex> g(mu_);
        auto it = live_.find(static_cast<char *>(ptr));
        if (it == live_.end()) return;
        char *a = it->first;
        Range r = it->second;
        live_.erase(it);
        in_use_ -= r.size;
        // merge with the following and the preceding free range of the slab
        auto nx = free_by_addr_.find(a + r.size);
        if (nx != free_by_addr_.end() && nx->second.slab == r.slab) {
            erase_size(nx->second.size, nx->first);
            r.size += nx->second.size;
            free_by_addr_.erase(nx);
        }
        auto pv = free_by_addr_.lower_bound(a);
        if (pv != free_by_addr_.begin()) {
            --pv;
            if (pv->second.slab == r.slab && pv->first + pv->second.size == a) {
                erase_size(pv->second.size, pv->first);
                a = pv->first;
                r.size += pv->second.size;
                free_by_addr_.erase(pv);
            }
        }
        insert_free(a, r);
    }

    // Frees every slab when no buffer is live (true if it did), so that the
    // next allocation starts a fresh slab that holds it.
    bool release_if_idle()
    {
        {
            std::lock_guard<std::mutex> g(mu_);
            if (!live_.empty() || slabs_.empty()) return false;
        }
        release();
        return true;
    }

    void release()
    {
        std::lock_guard<std::mutex> g(mu_);
        for (auto &s : slabs_) Backing::free(s.first);
        slabs_.clear();
        free_by_addr_.clear();
        free_by_size_.clear();
        live_.clear();
        reserved_ = in_use_ = 0;
    }

    struct Stats {
        size_t reserved, in_use, peak, slabs;
        long long device_allocs;
    };
    Stats stats()
    {
        std::lock_guard<std::mutex> g(mu_);
        return Stats{reserved_, in_use_, peak_, slabs_.size(), device_allocs_};
    }

private:
    struct Range {
        size_t slab;
        size_t size;
    };

    static size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

    bool grow_locked(size_t bytes)
    {
        device_allocs_++;
        void *p = Backing::alloc(bytes);
        if (!p) return false;
        slabs_.emplace_back(static_cast<char *>(p), bytes);
        reserved_ += bytes;
        insert_free(static_cast<char *>(p), Range{slabs_.size() - 1, bytes});
        return true;
    }

    void *take_locked(size_t n)
    {
        auto it = free_by_size_.lower_bound(n);
        if (it == free_by_size_.end()) return nullptr;
        char *a = it->second;
        free_by_size_.erase(it);
        auto fr = free_by_addr_.find(a);
        Range r = fr->second;
        free_by_addr_.erase(fr);
        if (r.size - n >= kAlign) insert_free(a + n, Range{r.slab, r.size - n});
        else n = r.size;
        live_[a] = Range{r.slab, n};
        return a;
    }

    void insert_free(char *a, Range r)
    {
        free_by_addr_[a] = r;
        free_by_size_.emplace(r.size, a);
    }

    void erase_size(size_t size, char *a)
    {
        auto rg = free_by_size_.equal_range(size);
        for (auto it = rg.first; it != rg.second; ++it)
            if (it->second == a) {
                free_by_size_.erase(it);
                return;
            }
    }

    std::mutex mu_;
    size_t cap_ = ~size_t(0);
    size_t reserved_ = 0, in_use_ = 0, peak_ = 0;
    long long device_allocs_ = 0;
    std::vector<std::pair<char *, size_t>> slabs_;
    std::map<char *, Range> free_by_addr_;
    std::multimap<size_t, char *> free_by_size_;
    std::unordered_map<char *, Range> live_;

public:
    // Bookkeeping check for tests: free ranges and live buffers tile every
    // slab exactly, free ranges are never adjacent, and the size index matches.
    bool consistent()
    {
        std::lock_guard<std::mutex> g(mu_);
        std::map<char *, std::pair<size_t, size_t>> all;  // start -> (slab, size)
        for (auto &kv : free_by_addr_) all[kv.first] = {kv.second.slab, kv.second.size};
        for (auto &kv : live_) {
            if (all.count(kv.first)) return false;
            all[kv.first] = {kv.second.slab, kv.second.size};
        }
        if (free_by_size_.size() != free_by_addr_.size()) return false;
        for (auto &kv : free_by_size_) {
            auto f = free_by_addr_.find(kv.second);
            if (f == free_by_addr_.end() || f->second.size != kv.first) return false;
        }
        size_t total = 0, used = 0;
        for (size_t k = 0; k < slabs_.size(); ++k) {
            char *a = slabs_[k].first;
            char *end = a + slabs_[k].second;
            bool prev_free = false;
            while (a < end) {
                auto it = all.find(a);
                if (it == all.end() || it->second.first != k) return false;
                const bool is_free = free_by_addr_.count(a) != 0;
                if (is_free && prev_free) return false;
                prev_free = is_free;
                if (!is_free) used += it->second.second;
                a += it->second.second;
            }
            if (a != end) return false;
            total += slabs_[k].second;
        }
        return total == reserved_ && used == in_use_;
    }
};

using Arena = ArenaT<>;

}  // namespace dwt
