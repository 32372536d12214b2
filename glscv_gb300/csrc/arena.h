// arena.h -- first-fit sub-allocator over one fixed device allocation.
//
// The serving loop reserves its whole HBM budget once and carves resident
// reference spectra and per-request workspaces out of it, so admission is a
// constant-time bookkeeping question ("does this request's workspace fit
// right now?") and no cudaMalloc/cudaFree happens while requests flow.
// Offsets are aligned to 256 bytes; freed ranges coalesce with neighbours.
// Not thread safe: the owner serialises calls.  Header-only and free of CUDA
// so its logic is unit-tested on the host.
#pragma once
#include <cstddef>
#include <cstdint>
#include <map>

namespace glsfft {

class Arena {
  public:
    static constexpr size_t kAlign = 256;
    static constexpr size_t kFail = SIZE_MAX;

    explicit Arena(size_t capacity = 0) { reset(capacity); }

    void reset(size_t capacity) {
        capacity_ = capacity / kAlign * kAlign;
        free_.clear();
        used_.clear();
        in_use_ = 0;
        if (capacity_) free_[0] = capacity_;
    }

    static size_t round_up(size_t n) { return (n + kAlign - 1) / kAlign * kAlign; }

    // Offset of a new block of at least n bytes, or kFail when none fits.
    size_t alloc(size_t n) {
        if (n == 0) n = 1;
        n = round_up(n);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                const size_t off = it->first, rest = it->second - n;
                free_.erase(it);
                if (rest) free_[off + n] = rest;
                used_[off] = n;
                in_use_ += n;
                return off;
            }
        }
        return kFail;
    }

    // Return a block; false for an offset that is not a live block.
    bool release(size_t off) {
        auto u = used_.find(off);
        if (u == used_.end()) return false;
        size_t start = off, len = u->second;
        used_.erase(u);
        in_use_ -= len;
        auto next = free_.lower_bound(start);
        if (next != free_.end() && next->first == start + len) {
            len += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == start) {
                start = prev->first;
                len += prev->second;
                free_.erase(prev);
            }
        }
        free_[start] = len;
        return true;
    }

    bool fits(size_t n) const {
        n = round_up(n ? n : 1);
        for (const auto &f : free_)
            if (f.second >= n) return true;
        return false;
    }

    size_t capacity() const { return capacity_; }
    size_t in_use() const { return in_use_; }
    size_t largest_free() const {
        size_t m = 0;
        for (const auto &f : free_) m = f.second > m ? f.second : m;
        return m;
    }
    size_t blocks() const { return used_.size(); }

  private:
    size_t capacity_ = 0, in_use_ = 0;
    std::map<size_t, size_t> free_;  // offset -> length
    std::map<size_t, size_t> used_;  // offset -> length
};

}  // namespace glsfft
