// mi_extents.h -- first-fit extent allocator over a fixed device pool (host
// code only).  The serving loop carves its HBM budget into one pool at
// start-up and gives every admitted request an extent of it; an extent returns
// to the pool when the request's results have left the device, so requests
// are admitted as soon as memory frees up, not batch by batch.
//
// Offsets and lengths are in floats.  Free extents are kept sorted by offset
// and merged with their neighbours on release, so the pool never fragments
// into pieces smaller than it must.
#pragma once

#include <cstdint>
#include <iterator>
#include <map>

namespace mi {

class ExtentPool {
public:
    explicit ExtentPool(int64_t floats) : size_(floats) {
        if (floats > 0) free_[0] = floats;
    }

    // First extent of `len` floats (len > 0) that fits, or -1 if none does.
    int64_t alloc(int64_t len) {
        if (len <= 0) return -1;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < len) continue;
            const int64_t off = it->first, rest = it->second - len;
            free_.erase(it);
            if (rest > 0) free_[off + len] = rest;
            used_ += len;
            if (used_ > peak_) peak_ = used_;
            return off;
        }
        return -1;
    }

    // Return [off, off + len) to the pool, merged with adjacent free extents.
    void release(int64_t off, int64_t len) {
        if (len <= 0) return;
        used_ -= len;
        auto next = free_.lower_bound(off);
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                off = prev->first;
                len += prev->second;
                free_.erase(prev);
            }
        }
        if (next != free_.end() && off + len == next->first) {
            len += next->second;
            free_.erase(next);
        }
        free_[off] = len;
    }

    int64_t size() const { return size_; }
    int64_t used() const { return used_; }
    int64_t peak() const { return peak_; }
    int64_t free_extents() const { return (int64_t)free_.size(); }
    // Largest single extent available now.
    int64_t largest_free() const {
        int64_t m = 0;
        for (const auto& f : free_) m = f.second > m ? f.second : m;
        return m;
    }

private:
    int64_t size_;
    int64_t used_ = 0, peak_ = 0;
    std::map<int64_t, int64_t> free_;   // offset -> length
};

}  // namespace mi
