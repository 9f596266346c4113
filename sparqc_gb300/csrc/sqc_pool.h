// First-fit allocator over one device allocation (host-side bookkeeping only): the serving
// loop carves per-circuit table slices and descriptor blocks out of one pool instead of
// calling cudaMalloc/cudaFree per request (which synchronize the device).
#pragma once
#include <cstddef>
#include <cstdint>
#include <map>

namespace sqc {

class RangePool {
public:
    // Manage [0, size); every block is aligned to `align` bytes (a power of two).
    void reset(size_t size, size_t align = 256) {
        free_.clear();
        align_ = align;
        size_ = size & ~(align - 1);
        if (size_) free_[0] = size_;
        used_ = 0;
    }
    // Offset of a free block of at least `bytes`, or SIZE_MAX.
    size_t alloc(size_t bytes) {
        const size_t need = (bytes + align_ - 1) & ~(align_ - 1);
        if (need == 0) return SIZE_MAX;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= need) {
                const size_t off = it->first, len = it->second;
                free_.erase(it);
                if (len > need) free_[off + need] = len - need;
                used_ += need;
                return off;
            }
        }
        return SIZE_MAX;
    }
    // Return a block (offset and the size it was allocated with); merges free neighbours.
    void release(size_t off, size_t bytes) {
        const size_t len = (bytes + align_ - 1) & ~(align_ - 1);
        used_ -= len;
        auto next = free_.lower_bound(off);
        size_t start = off, end = off + len;
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == start) {
                start = prev->first;
                free_.erase(prev);
            }
        }
        if (next != free_.end() && next->first == end) {
            end = next->first + next->second;
            free_.erase(next);
        }
        free_[start] = end - start;
    }
    size_t used() const { return used_; }
    size_t size() const { return size_; }
    size_t largest_free() const {
        size_t m = 0;
        for (auto& f : free_) m = f.second > m ? f.second : m;
        return m;
    }

private:
    std::map<size_t, size_t> free_;   // offset -> length
    size_t align_ = 256, size_ = 0, used_ = 0;
};

}  // namespace sqc
