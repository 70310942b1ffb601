// range_alloc.h -- first-fit allocator over [0, capacity) in element units,
// used by the server for the shape and pixel slots of its shared arenas.
// Plain host code (no CUDA): freed ranges merge with their neighbours, and
// growing the capacity frees the new tail.
#pragma once

#include <cstdint>
#include <iterator>
#include <map>

namespace ptgpu {

struct RangeAlloc {
    std::map<int64_t, int64_t> free_;   // start -> length
    int64_t capacity = 0;
    int64_t used = 0;
    // the lowest free range of at least n elements; false when none fits
    bool alloc(int64_t n, int64_t *start) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            *start = it->first;
            const int64_t rest = it->second - n, s = it->first + n;
            free_.erase(it);
            if (rest > 0) free_[s] = rest;
            used += n;
            return true;
        }
        return false;
    }
    void release(int64_t start, int64_t n) {
        used -= n;
        auto it = free_.emplace(start, n).first;
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
    // length of the free range that ends at the capacity (0 if the last
    // element is in use): growing by g makes a free range of free_tail() + g
    int64_t free_tail() const {
        if (free_.empty()) return 0;
        auto last = std::prev(free_.end());
        return last->first + last->second == capacity ? last->second : 0;
    }
    void grow(int64_t new_cap) {   // the new tail becomes free
        if (new_cap <= capacity) return;
        used += new_cap - capacity;   // release() below takes it off again
        release(capacity, new_cap - capacity);
        capacity = new_cap;
    }
};

}  // namespace ptgpu
