// Host-side test of the serving arena's bookkeeping (dwt_arena.h) over host
// memory: random allocation and release sequences keep every slab tiled
// exactly by live buffers and free ranges, live buffers never overlap, freed
// neighbours merge, the cap is respected, and releasing everything leaves one
// free range per slab.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <random>
#include <vector>

#include "../../libdwt_gb300/csrc/dwt_arena.h"

struct HostBacking {
    static long long live;
    static void *alloc(size_t bytes)
    {
        live++;
        return std::malloc(bytes);
    }
    static void free(void *p)
    {
        live--;
        std::free(p);
    }
};
long long HostBacking::live = 0;

#define CHECK(c)                                                        \
    do {                                                                \
        if (!(c)) {                                                     \
            std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
            return 1;                                                   \
        }                                                               \
    } while (0)

int main()
{
    {
        dwt::ArenaT<HostBacking> a;
        a.set_cap(size_t(64) << 20);
        CHECK(a.reserve(size_t(16) << 20));
        CHECK(a.stats().slabs == 1 && a.stats().reserved == (size_t(16) << 20));
        std::mt19937_64 rng(12345);
        std::map<char *, size_t> live;
        for (int it = 0; it < 20000; ++it) {
            const bool do_alloc = live.empty() || (rng() % 100) < 55;
            if (do_alloc) {
                // sizes log-uniform 1 B .. 4 MiB
                const double e = std::uniform_real_distribution<double>(0.0, 22.0)(rng);
                const size_t n = size_t(1) << int(e);
                char *p = static_cast<char *>(a.alloc(n));
                if (!p) {
                    // refused only when no free range fits and the cap leaves
                    // no room for a slab holding it
                    CHECK(a.stats().reserved + n > (size_t(64) << 20) || n > (size_t(1) << 30));
                    continue;
                }
                auto nx = live.lower_bound(p);
                if (nx != live.end()) CHECK(p + n <= nx->first);
                if (nx != live.begin()) {
                    auto pv = std::prev(nx);
                    CHECK(pv->first + pv->second <= p);
                }
                std::memset(p, 0x5a, n);
                live[p] = n;
            } else {
                auto itv = live.begin();
                std::advance(itv, rng() % live.size());
                a.free(itv->first);
                live.erase(itv);
            }
            if (it % 97 == 0) CHECK(a.consistent());
        }
        CHECK(a.consistent());
        CHECK(a.stats().reserved <= (size_t(64) << 20));
        for (auto &kv : live) a.free(kv.first);
        CHECK(a.consistent());
        CHECK(a.stats().in_use == 0);
        // everything released: one free range per slab, so a slab-sized
        // request fits again
        CHECK(a.alloc(size_t(16) << 20) != nullptr);
        CHECK(a.consistent());
        // beyond the cap: refused, nothing grows
        const size_t slabs = a.stats().slabs;
        CHECK(a.alloc(size_t(65) << 20) == nullptr);
        CHECK(a.stats().slabs == slabs);
    }
    CHECK(HostBacking::live == 0);
    std::printf("arena: ok\n");
    return 0;
}
