// fm_pool.h -- first-fit allocator of byte ranges with coalescing frees (host
// only).  The server leases level buffers and tables from the context's slab
// with it; the bookkeeping never touches the memory it manages.
#pragma once

#include <algorithm>
#include <cstdint>
#include <iterator>
#include <map>

namespace fm {

// Ranges of [0, size): first fit, neighbours merged on release.
class PoolAlloc {
public:
    void init(uint64_t size) {
        free_.clear();
        if (size) free_[0] = size;
        total_ = free_bytes_ = size;
        peak_ = 0;
    }
    bool alloc(uint64_t bytes, uint64_t& off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            off = it->first;
            const uint64_t rest = it->second - bytes;
            free_.erase(it);
            if (rest) free_[off + bytes] = rest;
            free_bytes_ -= bytes;
            peak_ = std::max(peak_, total_ - free_bytes_);
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t bytes) {
        free_bytes_ += bytes;
        auto next = free_.lower_bound(off);
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                off = prev->first;
                bytes += prev->second;
                free_.erase(prev);
            }
        }
        next = free_.lower_bound(off);
        if (next != free_.end() && off + bytes == next->first) {
            bytes += next->second;
            free_.erase(next);
        }
        free_[off] = bytes;
    }
    uint64_t largest() const {
        uint64_t m = 0;
        for (const auto& f : free_) m = std::max(m, f.second);
        return m;
    }
    uint64_t free_bytes() const { return free_bytes_; }
    uint64_t total() const { return total_; }
    uint64_t peak() const { return peak_; }
    size_t free_ranges() const { return free_.size(); }

private:
    std::map<uint64_t, uint64_t> free_;
    uint64_t total_ = 0, free_bytes_ = 0, peak_ = 0;
};

}  // namespace fm
