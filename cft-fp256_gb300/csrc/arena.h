// arena.h - first-fit allocation of byte offsets inside one device region
// (the serving loop's memory budget). Host-only bookkeeping: it never
// touches the region itself, so it is tested on its own without a GPU.
#pragma once
#include <algorithm>
#include <cstddef>
#include <iterator>
#include <map>

namespace cftg {

constexpr size_t ARENA_ALIGN = 256;
inline size_t round_up(size_t x) { return (std::max<size_t>(x, 1) + ARENA_ALIGN - 1) / ARENA_ALIGN * ARENA_ALIGN; }

// First-fit allocation of offsets inside one device region, free blocks
// coalesced on release.
class Arena {
public:
    void init(size_t bytes) { free_.clear(); free_[0] = bytes; size_ = bytes; }
    bool alloc(size_t bytes, size_t *off)
    {
        bytes = round_up(bytes);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const size_t o = it->first, rest = it->second - bytes;
            free_.erase(it);
            if (rest) free_[o + bytes] = rest;
            *off = o;
            used_ += bytes;
            peak_ = std::max(peak_, used_);
            return true;
        }
        return false;
    }
    void release(size_t off, size_t bytes)
    {
        bytes = round_up(bytes);
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t used() const { return used_; }
    size_t peak() const { return peak_; }
    size_t size() const { return size_; }
    size_t free_blocks() const { return free_.size(); }

private:
    std::map<size_t, size_t> free_;
    size_t size_ = 0, used_ = 0, peak_ = 0;
};

}  // namespace cftg
