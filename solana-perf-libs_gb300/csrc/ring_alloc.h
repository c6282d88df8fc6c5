// Allocation from a circular buffer in arrival order, with release in any
// order (host side, no CUDA).
//
// The served loop's resident signature service (server.cu) stages every
// request's inputs, results and chunk descriptors in rings sized when the
// server is created, so steady-state serving allocates nothing.  Requests
// are admitted in arrival order but complete in any order (a small request
// admitted after a large one finishes first), so space is reclaimed from the
// oldest live allocation onwards: an allocation's bytes become reusable once
// it and every allocation older than it have been released.
//
// Positions are virtual (a monotonic count of units); the physical offset is
// the virtual position modulo the capacity.  A contiguous allocation that
// would straddle the end of the buffer starts at the next lap instead; a
// non-contiguous one (chunk descriptors, addressed one by one modulo the
// ring size) may wrap.
//
// Tested on the host by tests/native/ring_alloc_check.cpp.
#pragma once
#include <stdint.h>

#include <algorithm>
#include <deque>

namespace gb300 {

class RingAlloc {
public:
    explicit RingAlloc(uint64_t cap = 0, bool contiguous = true) : cap_(cap), contiguous_(contiguous) {}

    void reset(uint64_t cap, bool contiguous = true) {
        cap_ = cap;
        contiguous_ = contiguous;
        tail_ = 0;
        next_id_ = 1;
        segs_.clear();
    }

    // Reserves n units aligned to `align` (a power of two that divides the
    // capacity, so virtual and physical alignment agree).  On success sets
    // *vpos (virtual start; physical start = *vpos % capacity) and *id (the
    // handle for release) and returns true; returns false when the space is
    // not free yet (or n exceeds the capacity, or align does not divide it).
    bool alloc(uint64_t n, uint64_t align, uint64_t* vpos, uint64_t* id) {
        if (cap_ == 0 || n > cap_ || align == 0 || cap_ % align) return false;
        uint64_t b = (tail_ + align - 1) & ~(align - 1);
        if (contiguous_ && n > 0 && (b % cap_) + n > cap_) b = (b / cap_ + 1) * cap_;
        const uint64_t oldest = segs_.empty() ? b : segs_.front().begin;
        if (b + n - oldest > cap_) return false;
        segs_.push_back({b, b + n, next_id_, false});
        tail_ = b + n;
        *vpos = b;
        *id = next_id_++;
        return true;
    }

    // Releases the allocation `id` (any order); returns false for an unknown id.
    bool release(uint64_t id) {
        auto it = std::lower_bound(segs_.begin(), segs_.end(), id,
                                   [](const Seg& s, uint64_t v) { return s.id < v; });
        if (it == segs_.end() || it->id != id || it->freed) return false;
        it->freed = true;
        while (!segs_.empty() && segs_.front().freed) segs_.pop_front();
        return true;
    }

    uint64_t capacity() const { return cap_; }
    bool empty() const { return segs_.empty(); }
    size_t live() const { return segs_.size(); }
    // units between the oldest live allocation and the end of the newest
    uint64_t span() const { return segs_.empty() ? 0 : tail_ - segs_.front().begin; }

private:
    struct Seg {
        uint64_t begin, end, id;
        bool freed;
    };
    uint64_t cap_;
    bool contiguous_;
    uint64_t tail_ = 0;
    uint64_t next_id_ = 1;
    std::deque<Seg> segs_;
};

}  // namespace gb300
