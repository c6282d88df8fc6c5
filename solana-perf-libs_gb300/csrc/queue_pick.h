// Which GPU and which of its queues serve a call (host side, no CUDA).
//
// The reference picks the next GPU in turn and, on it, the next queue in
// turn, then waits for that queue's lock (src/cuda-ecc-ed25519/gpu_ctx.cu:
// 46-73, the round-robin at :56-61).  Here the GPU is still the next in
// turn, but on it the call takes the first queue whose lock is free, and
// only when every queue is busy the next queue in turn, whose lock it then
// waits for.  A lone caller therefore keeps reusing one queue's device
// buffers and captured graphs, while concurrent callers still spread over
// the queues.
//
// The choice is kept apart from the CUDA runtime so that it can be tested
// on the host with any device count (tests/native/queue_pick_check.cpp).
#pragma once
#include <stdint.h>

namespace gb300 {

struct QueuePick {
    int gpu = -1;
    int queue = -1;
    bool held = false;      // true: the queue's lock is already taken by try_lock
};

template <int kMaxGpus>
struct QueueTurns {
    uint32_t next_gpu = 0;
    uint32_t next_queue[kMaxGpus] = {};
};

// Called with the pool's lock held.  try_lock(gpu, queue) attempts the
// queue's own lock without blocking.  When the result has held == false the
// caller must take the queue's lock itself, after releasing the pool's lock.
template <int kMaxGpus, class TryLock>
QueuePick pick_queue(QueueTurns<kMaxGpus>& turns, int num_gpus, int num_queues, TryLock&& try_lock) {
    QueuePick p;
    if (num_gpus <= 0 || num_queues <= 0) return p;
    p.gpu = (int)(turns.next_gpu % (uint32_t)num_gpus);
    turns.next_gpu++;
    for (int k = 0; k < num_queues; k++) {
        if (try_lock(p.gpu, k)) {
            p.queue = k;
            p.held = true;
            return p;
        }
    }
    p.queue = (int)(turns.next_queue[p.gpu] % (uint32_t)num_queues);
    turns.next_queue[p.gpu]++;
    return p;
}

}  // namespace gb300
