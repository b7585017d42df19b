// The serving budget's allocator (csrc/arena.h) under random traffic:
// allocations never overlap, stay inside the region and are 256-byte
// aligned; the in-use count matches; freeing everything coalesces the
// region back into one block. Prints "ok" or the first failure.
#include <cstdio>
#include <cstdint>
#include <map>
#include <random>
#include <vector>

#include "arena.h"

int main()
{
    const size_t region = size_t(1) << 30;
    cftg::Arena a;
    a.init(region);
    std::mt19937_64 rng(12345);
    std::map<size_t, size_t> live;                 // offset -> rounded size
    size_t used = 0;
    for (int step = 0; step < 200000; step++) {
        const bool do_alloc = live.empty() || (rng() % 100) < 55;
        if (do_alloc) {
            const size_t bytes = 1 + rng() % (size_t(1) << (8 + rng() % 17));
            size_t off = 0;
            if (!a.alloc(bytes, &off)) continue;
            const size_t sz = cftg::round_up(bytes);
            if (off % 256 || off + sz > region) { std::printf("outside or unaligned at %d\n", step); return 1; }
            auto nx = live.lower_bound(off);
            if (nx != live.end() && nx->first < off + sz) { std::printf("overlap after at %d\n", step); return 1; }
            if (nx != live.begin()) {
                auto pv = std::prev(nx);
                if (pv->first + pv->second > off) { std::printf("overlap before at %d\n", step); return 1; }
            }
            live[off] = sz;
            used += sz;
        } else {
            auto it = live.begin();
            std::advance(it, rng() % live.size());
            a.release(it->first, it->second);
            used -= it->second;
            live.erase(it);
        }
        if (a.used() != used) { std::printf("used %zu != %zu at %d\n", a.used(), used, step); return 1; }
    }
    for (auto &kv : live) a.release(kv.first, kv.second);
    if (a.used() != 0 || a.free_blocks() != 1) {
        std::printf("not coalesced: used %zu, %zu free blocks\n", a.used(), a.free_blocks());
        return 1;
    }
    size_t off = 0;
    if (!a.alloc(region, &off) || off != 0) { std::printf("whole region not allocatable\n"); return 1; }
    std::printf("ok\n");
    return 0;
}
