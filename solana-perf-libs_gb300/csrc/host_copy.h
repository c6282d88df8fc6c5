// Parallel copies of caller memory into page-locked staging (host side).
//
// A caller's pageable packet buffers go through the library's page-locked
// staging before one host-to-device copy, as in the reference
// (src/cuda-ecc-ed25519/gpu_ctx.cu:138-143).  One host thread moves that
// data at ~19 GB/s on the GB300's Grace host (131 MB in ~7 ms, as long as
// the batch's verify), while the memory system takes several times more, so
// large copies are split over a small pool of threads created on first use.
//
// One copy uses the pool at a time; a caller that finds it busy copies on
// its own thread.  Work is handed out in parts by a 64-bit ticket whose top
// half is the job's generation, so a worker that wakes late cannot claim a
// part of a newer job with an older job's description.
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <vector>

namespace gb300 {

struct CopyPiece {
    void* dst;
    const void* src;
    size_t len;
};

class CopyPool {
public:
    // Copies every piece (pieces must not overlap).
    static void copy(const CopyPiece* pc, size_t n) {
        size_t total = 0;
        for (size_t i = 0; i < n; i++) total += pc[i].len;
        if (total < kMinParallel) return serial(pc, n, 0, total);
        CopyPool& P = get();
        if (P.nthreads == 0 || !P.busy.try_lock()) return serial(pc, n, 0, total);
        P.run(pc, n, total);
        P.busy.unlock();
    }

private:
    static constexpr size_t kMinParallel = 4u << 20;   // below this one thread is as fast
    static constexpr size_t kPart = 1u << 20;          // smallest part

    struct Job {
        const CopyPiece* pc = nullptr;
        size_t n = 0, total = 0;
        uint32_t parts = 0, gen = 0;
    };

    std::mutex busy;                   // one job in the pool at a time
    std::mutex mu;
    std::condition_variable cv, cv_done;
    Job job;
    std::atomic<uint64_t> ticket{0};   // gen << 32 | next part
    std::atomic<uint32_t> remaining{0};
    uint32_t gen = 0;
    int nthreads = 0;

    static CopyPool& get() {
        // never destroyed: the workers wait on it until the process exits
        static CopyPool* p = new CopyPool();
        return *p;
    }

    CopyPool() {
        unsigned hw = std::thread::hardware_concurrency();
        int want = hw > 1 ? (int)(hw < 8 ? hw : 8) - 1 : 0;    // the caller is the 8th
        if (const char* v = getenv("GB300_CRYPT_COPY_THREADS")) want = atoi(v) - 1;
        if (want < 0) want = 0;
        if (want > 63) want = 63;
        for (int i = 0; i < want; i++) {
            try {
                std::thread(&CopyPool::worker, this).detach();
                nthreads++;
            } catch (...) {
                break;
            }
        }
    }

    // bytes [lo, hi) of the concatenation of the pieces
    static void serial(const CopyPiece* pc, size_t n, size_t lo, size_t hi) {
        size_t base = 0;
        for (size_t i = 0; i < n && base < hi; i++) {
            const size_t a = base, b = base + pc[i].len;
            base = b;
            if (b <= lo) continue;
            const size_t s = lo > a ? lo - a : 0, e = (hi < b ? hi : b) - a;
            if (e > s) memcpy(static_cast<uint8_t*>(pc[i].dst) + s, static_cast<const uint8_t*>(pc[i].src) + s, e - s);
        }
    }

    // claims and copies parts of job j while its generation is current
    void drain(const Job& j) {
        for (;;) {
            uint64_t cur = ticket.load();
            if ((uint32_t)(cur >> 32) != j.gen || (uint32_t)cur >= j.parts) return;
            if (!ticket.compare_exchange_weak(cur, cur + 1)) continue;
            const uint32_t p = (uint32_t)cur;
            serial(j.pc, j.n, j.total * p / j.parts, j.total * (p + 1) / j.parts);
            if (remaining.fetch_sub(1) == 1) {
                std::lock_guard<std::mutex> lk(mu);
                cv_done.notify_all();
            }
        }
    }

    void run(const CopyPiece* pc, size_t n, size_t total) {
        size_t parts = total / kPart;
        const size_t most = 4 * (size_t)(nthreads + 1);
        if (parts > most) parts = most;
        Job j;
        {
            std::lock_guard<std::mutex> lk(mu);
            j.pc = pc;
            j.n = n;
            j.total = total;
            j.parts = (uint32_t)parts;
            j.gen = ++gen;
            job = j;
            remaining.store(j.parts);
            ticket.store((uint64_t)j.gen << 32);
        }
        cv.notify_all();
        drain(j);
        std::unique_lock<std::mutex> lk(mu);
        cv_done.wait(lk, [&] { return remaining.load() == 0; });
    }

    void worker() {
        uint32_t seen = 0;
        for (;;) {
            Job j;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return gen != seen; });
                seen = gen;
                j = job;
            }
            drain(j);
        }
    }
};

}  // namespace gb300
