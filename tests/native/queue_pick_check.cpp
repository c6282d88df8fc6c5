// Checks gb300::pick_queue (solana-perf-libs_gb300/csrc/queue_pick.h), the
// library's choice of GPU and queue for each call, on the host with a faked
// device count, using real mutexes for the queue locks as the library does:
//   1. one caller, calls one after another: GPUs in turn, always the GPU's
//      first queue (the warm one);
//   2. concurrent callers that hold their queues: spread evenly over the
//      GPUs, never two on one queue while free queues remain;
//   3. more concurrent callers than queues on one GPU: the extra callers
//      wait on busy queues in turn and proceed when they are released, with
//      no two callers inside one queue at a time;
//   4. no GPU: no pick.
// Prints "ok" and exits 0 on success.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <mutex>
#include <thread>
#include <vector>

#include "queue_pick.h"

namespace {

constexpr int kMaxGpus = 8, kQueues = 8;

struct Pool {
    std::mutex mu;
    std::mutex q[kMaxGpus][kQueues];
    std::atomic<int> inside[kMaxGpus][kQueues];
    gb300::QueueTurns<kMaxGpus> turns;
    int num_gpus;
    explicit Pool(int n) : num_gpus(n) {
        for (auto& g : inside)
            for (auto& x : g) x = 0;
    }
    // the library's acquire(): pick under the pool lock, then lock the queue
    gb300::QueuePick acquire() {
        std::unique_lock<std::mutex> lk(mu);
        gb300::QueuePick p = gb300::pick_queue(turns, num_gpus, kQueues, [&](int g, int k) { return q[g][k].try_lock(); });
        lk.unlock();
        if (p.gpu >= 0 && !p.held) q[p.gpu][p.queue].lock();
        return p;
    }
    void release(const gb300::QueuePick& p) { q[p.gpu][p.queue].unlock(); }
};

bool fail(const char* what, int a, int b) {
    printf("FAIL %s (%d, %d)\n", what, a, b);
    return false;
}

bool sequential_calls() {
    for (int n = 1; n <= kMaxGpus; n++) {
        Pool P(n);
        for (int call = 0; call < 5 * n; call++) {
            gb300::QueuePick p = P.acquire();
            if (p.gpu != call % n) return fail("sequential: GPU not in turn", n, call);
            if (p.queue != 0 || !p.held) return fail("sequential: not the first idle queue", n, call);
            P.release(p);
        }
    }
    return true;
}

// `callers` threads each acquire a queue and hold it until all have one
bool concurrent_spread(int n, int callers) {
    Pool P(n);
    std::vector<gb300::QueuePick> got(callers);
    std::mutex m;
    std::condition_variable cv;
    int have = 0;
    std::vector<std::thread> th;
    for (int c = 0; c < callers; c++)
        th.emplace_back([&, c] {
            got[c] = P.acquire();
            std::unique_lock<std::mutex> lk(m);
            have++;
            cv.notify_all();
            cv.wait(lk, [&] { return have == callers; });
            lk.unlock();
            P.release(got[c]);
        });
    for (auto& t : th) t.join();
    std::vector<int> per_gpu(n, 0);
    std::vector<std::vector<int>> per_queue(n, std::vector<int>(kQueues, 0));
    for (auto& p : got) {
        if (p.gpu < 0 || p.gpu >= n || p.queue < 0 || p.queue >= kQueues) return fail("spread: bad pick", p.gpu, p.queue);
        per_gpu[p.gpu]++;
        per_queue[p.gpu][p.queue]++;
    }
    for (int g = 0; g < n; g++) {
        const int want = callers / n + (g < callers % n ? 1 : 0);
        if (per_gpu[g] != want) return fail("spread: GPU share", g, per_gpu[g]);
        for (int k = 0; k < kQueues; k++)
            if (per_queue[g][k] > 1) return fail("spread: two callers on one queue", g, k);
    }
    return true;
}

bool oversubscribed(int callers) {
    Pool P(1);
    std::atomic<int> max_inside{0}, done{0};
    std::vector<std::thread> th;
    for (int c = 0; c < callers; c++)
        th.emplace_back([&] {
            for (int rep = 0; rep < 50; rep++) {
                gb300::QueuePick p = P.acquire();
                const int now = ++P.inside[p.gpu][p.queue];
                int m = max_inside.load();
                while (now > m && !max_inside.compare_exchange_weak(m, now)) {
                }
                std::this_thread::sleep_for(std::chrono::microseconds(50));
                --P.inside[p.gpu][p.queue];
                P.release(p);
            }
            done++;
        });
    for (auto& t : th) t.join();
    if (done != callers) return fail("oversubscribed: callers lost", done.load(), callers);
    if (max_inside != 1) return fail("oversubscribed: a queue shared at once", max_inside.load(), 0);
    return true;
}

bool no_gpu() {
    Pool P(0);
    gb300::QueuePick p = P.acquire();
    return p.gpu < 0 ? true : fail("no GPU: got a pick", p.gpu, p.queue);
}

}  // namespace

int main() {
    bool ok = sequential_calls() && no_gpu();
    for (int n : {1, 2, 3, 8})
        for (int callers : {1, 5, 8, 16})
            if (callers <= n * kQueues) ok = ok && concurrent_spread(n, callers);
    ok = ok && oversubscribed(12) && oversubscribed(3);
    if (!ok) return 1;
    printf("ok\n");
    return 0;
}
