// Served request loop (include/gb300_serve.h): continuous batching of
// Ed25519 verify/sign jobs and PoH batches on one GPU.
//
// One dispatcher thread per server:
//   * completion: for every busy slot whose event has fired, copy each
//     request's results out of the slot's page-locked output, mark its ticket
//     done and return the slot's device bytes to the admission budget;
//   * admission: while a signature slot is free, take queued verify/sign
//     jobs in arrival order until the launch's item cap or the memory budget
//     would be exceeded, and run them as ONE persistent launch (the mixed
//     kernel of sig_batch.cu) on that slot's high-priority stream.  Queued
//     wire-format packet batches of one stride merge the same way into one
//     parse + verify + reduce launch (packets.cu), whose signature count is
//     known only on the device; a launch holds one of the two kinds.  PoH
//     batches run on low-priority streams (persistent PoH kernel);
//   * sleep on a condition variable when there is nothing to do (woken by
//     submissions; polls the GPU every 20 us while work is in flight).
// Slot buffers (device rings and page-locked staging) are sized at creation
// and stay resident, as do the basepoint tables; merged launches are kept
// within a slot's ring, so steady-state serving never allocates (a single
// request larger than a ring grows it with the stream-ordered allocator).
//
// Verify/sign jobs (offset form) go by default to the resident signature
// service instead (sig_service.cu): the submitting thread stages the job
// into rings allocated at creation, copies its inputs to the GPU and
// publishes its 32-item chunks to the FIFO of a long-lived kernel; the
// dispatcher returns each request as soon as the GPU has written its
// completion word, independently of what else is in flight, and launches
// the kernel again whenever requests are waiting and it has left.  A job
// too large for the rings takes the slot path.
#include <cuda.h>            // driver types of the stream write (the driver library is not linked)
#include <cuda_runtime.h>
#include <sys/prctl.h>

#include <chrono>
#include <climits>
#include <condition_variable>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "ed25519.h"
#include "gb300_serve.h"
#include "host_buffers.h"
#include "host_copy.h"
#include "kernels.h"
#include "ring_alloc.h"
#include "tables.cuh"

namespace {

using gb300::DevBuf;
using gb300::HostBuf;
using gb300::round_up;

bool page_locked(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

struct Req {
    uint64_t ticket = 0;
    int kind = 0;                 // 0 verify, 1 sign, 2 poh, 3 wire packets
    gb300_sig_job job{};
    uint8_t* hashes = nullptr;
    const uint64_t* counts = nullptr;
    // wire packets: the caller's runs of packet slots (descriptors copied at
    // submission), data lengths and per-packet outputs
    std::vector<gpu_Elems> elems;
    uint32_t stride = 0;
    const uint32_t* lens = nullptr;
    uint8_t* pkt_out = nullptr;
    uint32_t* sig_counts = nullptr;
    uint64_t n = 0;               // items (signatures, entries or packets)
    uint64_t ring_bytes = 0;      // packet bytes in the slot's ring
    bool locked = false;          // packet bytes page-locked (checked at submission)
    uint64_t bytes = 0;           // device bytes while in flight
};

struct Slot {
    int64_t t_admit = 0, t_enqueued = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    // timed GPU phases of the launch: ev_in (inputs start copying), ev_run
    // (kernels start), ev_out (results start copying), done (all copied)
    cudaEvent_t ev_in = nullptr, ev_run = nullptr, ev_out = nullptr;
    bool busy = false;
    int kind = 0;                 // 0 signatures, 2 PoH, 3 wire packets
    DevBuf d_data, d_index, d_out, d_scratch;
    HostBuf h_stage, h_out;
    std::vector<Req> reqs;
    uint64_t bytes = 0;
    uint64_t nv = 0, ns = 0, sig_out_off = 0, poh_n = 0;
    cudaError_t err = cudaSuccess;
};

// ---- resident signature service: host state --------------------------------

constexpr uint32_t kSvcMaxReq = 4096;              // request slots in flight
constexpr uint32_t kSvcRing = 1u << 18;            // chunk descriptors (4 MiB)
constexpr uint64_t kSvcStageBytes = 256ull << 20;  // page-locked staging: index arrays, pageable packets
constexpr uint64_t kSvcResultBytes = 64ull << 20;  // page-locked results the GPU writes
constexpr uint64_t kSvcDevBytes = 1ull << 30;      // device input ring (at most the memory cap)
constexpr uint32_t kPohYieldChunks = 64;           // PoH gives way at this many waiting chunks (0: never)
constexpr size_t kTraceCap = 16384;                // launch-trace entries kept (the oldest quarter goes when full)

typedef CUresult (*WriteValue32Fn)(CUstream, CUdeviceptr, cuuint32_t, unsigned int);

struct SvcInflight {
    uint64_t ticket;
    int kind;                    // 0 verify, 1 sign
    uint32_t slot, gen;
    uint64_t n;
    uint8_t* out;                // caller's output
    uint64_t out_bytes;
    const uint8_t* res;          // the results in the page-locked ring
    uint64_t id_dev, id_stage, id_res, id_chunk;
    uint64_t dev_bytes;
    int64_t t_pub;
};

struct SvcDone {
    uint64_t ticket, n;
    int status;                  // 1 done, < 0 error
    int64_t t_pub, t_done;
    float wait_ms, run_ms;       // GPU: publication to first claimed chunk, first claim to completion
};

struct SigService {
    bool on = false;
    std::mutex mu;               // ring allocation and the order of copies and publications
    cudaStream_t copy = nullptr, run = nullptr;
    cudaEvent_t run_done = nullptr;
    bool launched = false;
    SvcDevice* d_state = nullptr;
    uint32_t* d_items = nullptr;
    uint64_t* d_first = nullptr;
    uint8_t* d_in = nullptr;
    gb300::RingAlloc dev_ring, stage_ring, res_ring, chunks;
    uint8_t* h_stage = nullptr;
    uint8_t* h_res = nullptr;
    uint8_t* d_res = nullptr;
    void* h_ctl = nullptr;       // mapped: request table, chunk ring, completion words, times
    SvcReq* h_req = nullptr;
    SvcChunk* h_ring = nullptr;
    uint32_t* h_done = nullptr;
    uint64_t* h_times = nullptr; // [2 * kSvcMaxReq]: first claim, completion (%globaltimer)
    int64_t clock_offset = 0;    // host steady-clock ns minus %globaltimer ns
    SvcParams params{};
    uint64_t chunk_tail = 0;     // chunks published (virtual count; the GPU sees the low 32 bits)
    std::vector<uint32_t> free_slots, gen;
    std::vector<SvcInflight> inflight;
    std::deque<Req> pending;     // admitted in arrival order as ring space frees up
    uint64_t in_use = 0;         // device bytes of the requests in flight
    WriteValue32Fn write_value = nullptr;
    int blocks_per_sm = 2;
    uint64_t launches = 0, max_inflight = 0, served = 0, fallback = 0;
    cudaError_t err = cudaSuccess;
};

}  // namespace

struct gb300_server {
    int dev = -1;
    CryptDeviceInfo info{};
    uint64_t cap = 0, in_use = 0;
    uint32_t max_items = 0;
    int poh_form = kPohPackedSingle, poh_warps = 0;   // shape of the PoH launches
    PohYield poh_yield{};                               // with the signature service: its FIFO
    std::vector<Slot> sig_slots, poh_slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req> pending_sig, pending_poh;
    std::unordered_map<uint64_t, int> status;   // 0 pending, 1 done, < 0 error
    std::unordered_map<uint64_t, std::pair<int64_t, int64_t>> times;   // submit, completion (steady ns)
    uint64_t next_ticket = 1;
    bool stop = false;
    std::thread worker;
    // counters
    uint64_t launches_sig = 0, launches_poh = 0, requests_done = 0, merged_max = 0, items_done = 0;
    // per-launch timeline of the last launches: kind, requests, items,
    // admitted / enqueued / observed complete (steady ns)
    struct Trace {
        int kind;
        uint32_t reqs;
        uint64_t items;
        int64_t t_admit, t_enqueued, t_complete;
        float copy_in_ms, kernels_ms, copy_out_ms;   // GPU time of each phase (events)
    };
    std::vector<Trace> trace;
    SigService svc;
};

namespace {

int64_t now_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch()).count();
}

uint64_t sig_bytes(const gb300_sig_job& j) {
    return j.packets_len + 16ull * j.num + (j.kind == 0 ? j.num : 64ull * j.num) + 64;
}

// Output layout of a packets launch: verdicts, then signature counts.
uint64_t pkt_counts_off(uint64_t n) { return round_up(n, 256); }

// Stage and launch the requests in S.reqs (signature jobs) on S.stream.
cudaError_t launch_sigs(gb300_server* sv, Slot& S) {
    uint64_t nv = 0, ns = 0, total = 0;
    bool locked = true;
    for (auto& r : S.reqs) {
        (r.kind == 0 ? nv : ns) += r.n;
        total += r.job.packets_len;
        locked = locked && r.locked;
    }
    S.nv = nv;
    S.ns = ns;
    S.sig_out_off = round_up(nv, 64);
    const size_t idx_bytes = 16ull * (nv + ns), out_bytes = S.sig_out_off + 64ull * ns;
    const size_t pk_off = round_up(idx_bytes, 256);
    cudaError_t e;
    if ((e = S.d_data.ensure(total + 16, S.stream)) != cudaSuccess) return e;
    if ((e = S.d_index.ensure(idx_bytes, S.stream)) != cudaSuccess) return e;
    if ((e = S.d_out.ensure(out_bytes, S.stream)) != cudaSuccess) return e;
    if ((e = S.d_scratch.ensure(256, S.stream)) != cudaSuccess) return e;
    if ((e = S.h_stage.ensure(pk_off + (locked ? 0 : total))) != cudaSuccess) return e;
    if ((e = S.h_out.ensure(out_bytes)) != cudaSuccess) return e;
    uint32_t* hv = static_cast<uint32_t*>(S.h_stage.p);
    uint32_t* hs = hv + 4 * nv;
    uint8_t* img = static_cast<uint8_t*>(S.h_stage.p) + pk_off;
    uint8_t* dpk = static_cast<uint8_t*>(S.d_data.p);
    uint64_t base = 0, iv = 0, is = 0;
    std::vector<gb300::CopyPiece> pcs;
    if ((e = cudaEventRecord(S.ev_in, S.stream)) != cudaSuccess) return e;
    for (auto& r : S.reqs) {
        const gb300_sig_job& J = r.job;
        uint32_t* h = r.kind == 0 ? hv : hs;
        const uint64_t cnt = r.kind == 0 ? nv : ns;
        uint64_t& pos = r.kind == 0 ? iv : is;
        for (uint32_t i = 0; i < J.num; i++) {
            const uint64_t m = J.message_lens[i], po = J.public_key_offsets[i], ko = J.key_offsets[i],
                           mo = J.message_start_offsets[i];
            const bool ok = po + 32 <= J.packets_len && ko + 64 <= J.packets_len && mo + m <= J.packets_len;
            h[pos + i] = ok ? (uint32_t)m : 0xffffffffu;
            h[cnt + pos + i] = ok ? (uint32_t)(base + po) : 0u;
            h[2 * cnt + pos + i] = ok ? (uint32_t)(base + ko) : 0u;
            h[3 * cnt + pos + i] = ok ? (uint32_t)(base + mo) : 0u;
        }
        if (J.packets_len) {
            if (locked) {
                e = cudaMemcpyAsync(dpk + base, J.packets, J.packets_len, cudaMemcpyHostToDevice, S.stream);
                if (e != cudaSuccess) return e;
            } else {
                pcs.push_back({img + base, J.packets, J.packets_len});
            }
        }
        pos += J.num;
        base += J.packets_len;
    }
    gb300::CopyPool::copy(pcs.data(), pcs.size());
    if ((e = cudaMemcpyAsync(S.d_index.p, S.h_stage.p, idx_bytes, cudaMemcpyHostToDevice, S.stream)) != cudaSuccess)
        return e;
    if (!locked && total && (e = cudaMemcpyAsync(dpk, img, total, cudaMemcpyHostToDevice, S.stream)) != cudaSuccess)
        return e;
    const uint32_t* dv = static_cast<const uint32_t*>(S.d_index.p);
    const uint32_t* ds = dv + 4 * nv;
    uint8_t* dout = static_cast<uint8_t*>(S.d_out.p);
    SigWork w;
    w.v = SigBatch{dpk, total, dv, dv + nv, dv + 2 * nv, dv + 3 * nv, (uint32_t)nv, dout, sv->info.tables};
    w.v.window = sv->info.verify_window;
    w.s = SigBatch{dpk, total, ds, ds + ns, ds + 2 * ns, ds + 3 * ns, (uint32_t)ns, dout + S.sig_out_off,
                   sv->info.tables};
    w.sign_base = (uint32_t)((nv + 31) / 32 * 32);
    w.total_chunks = (uint32_t)((w.sign_base + ns + 31) / 32);
    w.next = static_cast<uint32_t*>(S.d_scratch.p);
    if ((e = cudaEventRecord(S.ev_run, S.stream)) != cudaSuccess) return e;
    if ((e = launch_sig_batch(w, sv->info.sig_threads, sv->info.sig_blocks_per_sm, sv->info.sms, S.stream)) !=
        cudaSuccess)
        return e;
    if ((e = cudaEventRecord(S.ev_out, S.stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(S.h_out.p, dout, out_bytes, cudaMemcpyDeviceToHost, S.stream)) != cudaSuccess) return e;
    return cudaEventRecord(S.done, S.stream);
}

// Stage and launch the wire-packet requests in S.reqs (one stride) on
// S.stream: packet slots into the ring (page-locked runs copied directly),
// data lengths beside them, then the device parse / verify / reduce.
cudaError_t launch_packets(gb300_server* sv, Slot& S) {
    const uint64_t stride = S.reqs.front().stride;
    uint64_t n = 0;
    bool locked = true;
    for (auto& r : S.reqs) {
        n += r.n;
        locked = locked && r.locked;
    }
    S.nv = n;
    const uint64_t total = n * stride, lens_bytes = 4 * n, pk_off = round_up(lens_bytes, 256);
    const uint64_t out_bytes = pkt_counts_off(n) + 4 * n;
    const size_t ws_bytes = packets_workspace_size((uint32_t)n, stride);
    cudaError_t e;
    if ((e = S.d_data.ensure(total + 16, S.stream)) != cudaSuccess) return e;
    if ((e = S.d_index.ensure(lens_bytes, S.stream)) != cudaSuccess) return e;
    if ((e = S.d_out.ensure(out_bytes, S.stream)) != cudaSuccess) return e;
    if ((e = S.d_scratch.ensure(ws_bytes, S.stream)) != cudaSuccess) return e;
    if ((e = S.h_stage.ensure(pk_off + (locked ? 0 : total))) != cudaSuccess) return e;
    if ((e = S.h_out.ensure(out_bytes)) != cudaSuccess) return e;
    uint32_t* hl = static_cast<uint32_t*>(S.h_stage.p);
    uint8_t* img = static_cast<uint8_t*>(S.h_stage.p) + pk_off;
    uint8_t* dpk = static_cast<uint8_t*>(S.d_data.p);
    uint64_t pos = 0;
    std::vector<gb300::CopyPiece> pcs;
    if ((e = cudaEventRecord(S.ev_in, S.stream)) != cudaSuccess) return e;
    for (auto& r : S.reqs) {
        memcpy(hl + pos, r.lens, 4 * r.n);
        uint64_t p = pos;
        for (const gpu_Elems& g : r.elems) {
            if (!g.num) continue;
            const uint64_t b = (uint64_t)g.num * stride;
            if (locked) {
                e = cudaMemcpyAsync(dpk + p * stride, g.elems, b, cudaMemcpyHostToDevice, S.stream);
                if (e != cudaSuccess) return e;
            } else {
                pcs.push_back({img + p * stride, g.elems, b});
            }
            p += g.num;
        }
        pos += r.n;
    }
    gb300::CopyPool::copy(pcs.data(), pcs.size());
    if ((e = cudaMemcpyAsync(S.d_index.p, hl, lens_bytes, cudaMemcpyHostToDevice, S.stream)) != cudaSuccess)
        return e;
    if (!locked && (e = cudaMemcpyAsync(dpk, img, total, cudaMemcpyHostToDevice, S.stream)) != cudaSuccess)
        return e;
    uint8_t* dout = static_cast<uint8_t*>(S.d_out.p);
    if ((e = cudaEventRecord(S.ev_run, S.stream)) != cudaSuccess) return e;
    if ((e = launch_packets_verify(dpk, stride, (uint32_t)n, static_cast<const uint32_t*>(S.d_index.p),
                                   S.d_scratch.p, S.d_scratch.cap, dout,
                                   reinterpret_cast<uint32_t*>(dout + pkt_counts_off(n)), sv->info.tables,
                                   sv->info.sig_threads, sv->info.sig_blocks_per_sm, sv->info.sms, S.stream,
                                   sv->info.verify_window)) != cudaSuccess)
        return e;
    if ((e = cudaEventRecord(S.ev_out, S.stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(S.h_out.p, dout, out_bytes, cudaMemcpyDeviceToHost, S.stream)) != cudaSuccess) return e;
    return cudaEventRecord(S.done, S.stream);
}

cudaError_t launch_pohs(gb300_server* sv, Slot& S) {
    uint64_t n = 0;
    for (auto& r : S.reqs) n += r.n;
    S.poh_n = n;
    const size_t hb = 32ull * n, cb = 8ull * n;
    cudaError_t e;
    if ((e = S.d_data.ensure(hb + cb, S.stream)) != cudaSuccess) return e;
    if ((e = S.d_scratch.ensure(poh_batch_workspace_size(n), S.stream)) != cudaSuccess) return e;
    if ((e = S.h_stage.ensure(hb + cb)) != cudaSuccess) return e;
    uint8_t* st = static_cast<uint8_t*>(S.h_stage.p);
    uint64_t pos = 0;
    for (auto& r : S.reqs) {
        memcpy(st + 32 * pos, r.hashes, 32ull * r.n);
        memcpy(st + hb + 8 * pos, r.counts, 8ull * r.n);
        pos += r.n;
    }
    uint8_t* d = static_cast<uint8_t*>(S.d_data.p);
    if ((e = cudaEventRecord(S.ev_in, S.stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(d, st, hb + cb, cudaMemcpyHostToDevice, S.stream)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(S.ev_run, S.stream)) != cudaSuccess) return e;
    if ((e = launch_poh_batch(d, reinterpret_cast<const uint64_t*>(d + hb), n, S.d_scratch.p, sv->poh_warps,
                              S.stream, sv->poh_form, sv->poh_yield.chunks ? &sv->poh_yield : nullptr)) != cudaSuccess)
        return e;
    if ((e = cudaEventRecord(S.ev_out, S.stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(st, d, hb, cudaMemcpyDeviceToHost, S.stream)) != cudaSuccess) return e;
    return cudaEventRecord(S.done, S.stream);
}

// Results of a finished slot back to the callers (dispatcher thread, no lock held).
void deliver(Slot& S) {
    if (S.kind == 0) {
        const uint8_t* ho = static_cast<const uint8_t*>(S.h_out.p);
        uint64_t ov = 0, os = 0;
        for (auto& r : S.reqs) {
            if (r.kind == 0) {
                if (S.err == cudaSuccess) memcpy(r.job.out, ho + ov, r.n);
                else memset(r.job.out, 0, r.n);
                ov += r.n;
            } else {
                if (S.err == cudaSuccess) memcpy(r.job.out, ho + S.sig_out_off + 64 * os, 64ull * r.n);
                else memset(r.job.out, 0, 64ull * r.n);
                os += r.n;
            }
        }
    } else if (S.kind == 3) {
        const uint8_t* ho = static_cast<const uint8_t*>(S.h_out.p);
        const uint32_t* hc = reinterpret_cast<const uint32_t*>(ho + pkt_counts_off(S.nv));
        uint64_t pos = 0;
        for (auto& r : S.reqs) {
            if (S.err == cudaSuccess) {
                memcpy(r.pkt_out, ho + pos, r.n);
                if (r.sig_counts) memcpy(r.sig_counts, hc + pos, 4 * r.n);
            } else {
                memset(r.pkt_out, 0, r.n);
                if (r.sig_counts) memset(r.sig_counts, 0, 4 * r.n);
            }
            pos += r.n;
        }
    } else if (S.err == cudaSuccess) {
        const uint8_t* st = static_cast<const uint8_t*>(S.h_stage.p);
        uint64_t pos = 0;
        for (auto& r : S.reqs) {
            memcpy(r.hashes, st + 32 * pos, 32ull * r.n);
            pos += r.n;
        }
    }
}

// ---- resident signature service: host side --------------------------------

// Publishes chunks [0, tail) to the service kernel: a stream write ordered
// after the inputs' copies on the same stream (preceded by a system-wide
// fence).  Without the driver entry point, a one-thread kernel does the same.
__global__ void svc_publish_kernel(uint32_t* tail, uint32_t v) {
    __threadfence_system();
    *reinterpret_cast<volatile uint32_t*>(tail) = v;
}

cudaError_t svc_publish(SigService& V, uint32_t tail) {
    if (V.write_value) {
        const CUresult r = V.write_value(reinterpret_cast<CUstream>(V.copy),
                                         reinterpret_cast<CUdeviceptr>(&V.d_state->tail), tail, 0);
        if (r == CUDA_SUCCESS) return cudaSuccess;
        V.write_value = nullptr;                 // not supported here: the kernel from now on
    }
    svc_publish_kernel<<<1, 1, 0, V.copy>>>(&V.d_state->tail, tail);
    return cudaGetLastError();
}

uint64_t env_mib(const char* name, uint64_t dflt) {
    const char* v = getenv(name);
    return v && atoi(v) > 0 ? (uint64_t)atoi(v) << 20 : dflt;
}

bool svc_create(gb300_server* sv) {
    SigService& V = sv->svc;
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    const uint64_t dev_bytes = std::min<uint64_t>(env_mib("GB300_CRYPT_SERVER_SVC_DEVICE_MB", kSvcDevBytes),
                                                  round_up(sv->cap, 1ull << 20));
    const uint64_t stage_bytes = env_mib("GB300_CRYPT_SERVER_SVC_STAGE_MB", kSvcStageBytes);
    const uint64_t result_bytes = env_mib("GB300_CRYPT_SERVER_SVC_RESULT_MB", kSvcResultBytes);
    const size_t ctl = sizeof(SvcReq) * kSvcMaxReq + sizeof(SvcChunk) * kSvcRing + 4ull * kSvcMaxReq +
                       16ull * kSvcMaxReq;
    bool ok = cudaStreamCreateWithPriority(&V.copy, cudaStreamNonBlocking, hi) == cudaSuccess &&
              cudaStreamCreateWithPriority(&V.run, cudaStreamNonBlocking, hi) == cudaSuccess &&
              cudaEventCreateWithFlags(&V.run_done, cudaEventDisableTiming) == cudaSuccess &&
              cudaMalloc(&V.d_state, sizeof(SvcDevice)) == cudaSuccess &&
              cudaMalloc(&V.d_items, 4ull * kSvcMaxReq) == cudaSuccess &&
              cudaMalloc(&V.d_first, 8ull * kSvcMaxReq) == cudaSuccess &&
              cudaMalloc(&V.d_in, dev_bytes) == cudaSuccess &&
              cudaHostAlloc(&V.h_stage, stage_bytes, cudaHostAllocDefault) == cudaSuccess &&
              cudaHostAlloc(&V.h_res, result_bytes, cudaHostAllocMapped) == cudaSuccess &&
              cudaHostAlloc(&V.h_ctl, ctl, cudaHostAllocMapped) == cudaSuccess;
    void *d_res = nullptr, *d_ctl = nullptr;
    ok = ok && cudaHostGetDevicePointer(&d_res, V.h_res, 0) == cudaSuccess &&
         cudaHostGetDevicePointer(&d_ctl, V.h_ctl, 0) == cudaSuccess;
    ok = ok && cudaMemsetAsync(V.d_state, 0, sizeof(SvcDevice), V.copy) == cudaSuccess &&
         cudaMemsetAsync(V.d_items, 0, 4ull * kSvcMaxReq, V.copy) == cudaSuccess &&
         cudaMemsetAsync(V.d_first, 0xff, 8ull * kSvcMaxReq, V.copy) == cudaSuccess &&
         cudaStreamSynchronize(V.copy) == cudaSuccess;
    if (!ok) return false;
    memset(V.h_ctl, 0, ctl);
    V.d_res = static_cast<uint8_t*>(d_res);
    V.h_req = static_cast<SvcReq*>(V.h_ctl);
    V.h_ring = reinterpret_cast<SvcChunk*>(V.h_req + kSvcMaxReq);
    V.h_done = reinterpret_cast<uint32_t*>(V.h_ring + kSvcRing);
    V.h_times = reinterpret_cast<uint64_t*>(V.h_done + kSvcMaxReq);
    auto* dreq = static_cast<SvcReq*>(d_ctl);
    auto* dring = reinterpret_cast<SvcChunk*>(dreq + kSvcMaxReq);
    V.dev_ring.reset(dev_bytes);
    V.stage_ring.reset(stage_bytes);
    V.res_ring.reset(result_bytes);
    V.chunks.reset(kSvcRing, false);
    V.free_slots.resize(kSvcMaxReq);
    for (uint32_t k = 0; k < kSvcMaxReq; k++) V.free_slots[k] = kSvcMaxReq - 1 - k;
    V.gen.assign(kSvcMaxReq, 0);
    V.params.dev = V.d_state;
    V.params.items_done = V.d_items;
    V.params.req = dreq;
    V.params.ring = dring;
    V.params.done = reinterpret_cast<uint32_t*>(dring + kSvcRing);
    V.params.first_claim = V.d_first;
    V.params.times = reinterpret_cast<uint64_t*>(V.params.done + kSvcMaxReq);
    V.params.ring_size = kSvcRing;
    const char* idle = getenv("GB300_CRYPT_SERVER_IDLE_US");
    V.params.idle_ns = 1000ull * (uint64_t)(idle && atoi(idle) > 0 ? atoi(idle) : 20000);
    V.params.tables = sv->info.tables;
    V.params.first_warps = 4u * (uint32_t)sv->info.sms;
    if (poh_round_warp_map(&V.params.poh_slots, &V.params.poh_busy_slots) != cudaSuccess) return false;
    if (const char* b = getenv("GB300_CRYPT_SERVER_SVC_BLOCKS")) V.blocks_per_sm = atoi(b) > 0 ? atoi(b) : 2;
    // PoH launches give way while this many chunks wait unclaimed (PohYield)
    sv->poh_yield.head = &V.d_state->head;
    sv->poh_yield.tail = &V.d_state->tail;
    sv->poh_yield.chunks = kPohYieldChunks;
    if (const char* y = getenv("GB300_CRYPT_SERVER_POH_YIELD")) sv->poh_yield.chunks = (uint32_t)std::max(0, atoi(y));
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuStreamWriteValue32", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        V.write_value = reinterpret_cast<WriteValue32Fn>(fn);
    cudaGetLastError();
    if (load_kernels(svc_publish_kernel) != cudaSuccess) return false;
    // the GPU clock against the host's: the best of a few round trips
    {
        int64_t best = INT64_MAX;
        for (int k = 0; k < 5; k++) {
            const int64_t t0 = now_ns();
            if (launch_svc_clock(V.params.times, V.copy) != cudaSuccess ||
                cudaStreamSynchronize(V.copy) != cudaSuccess)
                return false;
            const int64_t t1 = now_ns();
            if (t1 - t0 < best) {
                best = t1 - t0;
                V.clock_offset = (t0 + t1) / 2 - (int64_t)__atomic_load_n(&V.h_times[0], __ATOMIC_ACQUIRE);
            }
        }
        V.h_times[0] = 0;
    }
    V.on = true;
    return true;
}

void svc_destroy(gb300_server* sv) {
    SigService& V = sv->svc;
    if (V.copy && V.d_state) {
        // warps leave as soon as the FIFO is empty (everything published is done by now)
        const uint32_t one = 1;
        cudaMemcpyAsync(&V.d_state->stop, &one, 4, cudaMemcpyHostToDevice, V.copy);
        cudaStreamSynchronize(V.copy);
    }
    if (V.run) cudaStreamSynchronize(V.run);
    if (V.copy) cudaStreamSynchronize(V.copy);
    if (V.d_state) cudaFree(V.d_state);
    if (V.d_items) cudaFree(V.d_items);
    if (V.d_first) cudaFree(V.d_first);
    if (V.d_in) cudaFree(V.d_in);
    if (V.h_stage) cudaFreeHost(V.h_stage);
    if (V.h_res) cudaFreeHost(V.h_res);
    if (V.h_ctl) cudaFreeHost(V.h_ctl);
    if (V.run_done) cudaEventDestroy(V.run_done);
    if (V.run) cudaStreamDestroy(V.run);
    if (V.copy) cudaStreamDestroy(V.copy);
    cudaGetLastError();
    V.on = false;
}

// The kernel is running, or launched now when it has left and requests are
// waiting on it (V.mu held).
void svc_ensure_running(gb300_server* sv) {
    SigService& V = sv->svc;
    if (V.inflight.empty() || V.err != cudaSuccess) return;
    if (V.launched) {
        const cudaError_t q = cudaEventQuery(V.run_done);
        if (q == cudaErrorNotReady) return;
        if (q != cudaSuccess) {
            V.err = q;
            return;
        }
    }
    // the launch's exit flag and claim time start from zero (stream order:
    // after the previous launch has left)
    cudaError_t e = cudaMemsetAsync(&V.d_state->exiting, 0,
                                    offsetof(SvcDevice, warps) - offsetof(SvcDevice, exiting), V.run);
    if (e == cudaSuccess) e = cudaMemsetAsync(V.d_state->sm_blocks, 0, sizeof(V.d_state->sm_blocks), V.run);
    if (e == cudaSuccess) e = launch_sig_service(V.params, V.blocks_per_sm, sv->info.sms, V.run);
    if (e == cudaSuccess) e = cudaEventRecord(V.run_done, V.run);
    if (e != cudaSuccess) {
        V.err = e;
        return;
    }
    V.launched = true;
    V.launches++;
}

// Stages and publishes one verify/sign job (V.mu held).  1: published; 0: the
// rings have no room now (retry after completions); -1: it never fits the
// rings (take the slot path).
int svc_try_submit(gb300_server* sv, const Req& r) {
    SigService& V = sv->svc;
    const gb300_sig_job& J = r.job;
    const uint64_t n = r.n;
    const bool verify = r.kind == 0;
    // four lanes per signature while the verifies in flight leave the GPU
    // idle (the size rule of the one-call form: up to 64 per SM);
    // GB300_CRYPT_VERIFY_FORM = 0 / 1 forces one form, as everywhere
    static const int forced = getenv("GB300_CRYPT_VERIFY_FORM") ? atoi(getenv("GB300_CRYPT_VERIFY_FORM")) : -1;
    uint64_t v_inflight = 0;
    for (const SvcInflight& f : V.inflight)
        if (f.kind == 0) v_inflight += f.n;
    const bool quad = verify && (forced == kVerifyQuad ||
                                 (forced != kVerifySingle && v_inflight + n <= 64ull * (uint64_t)sv->info.sms));
    const uint32_t per = quad ? 8u : 32u;
    const uint64_t nchunks = (n + per - 1) / per;
    const uint64_t idx_bytes = 16 * n, pk_off = round_up(idx_bytes, 256);
    const uint64_t dev_need = pk_off + J.packets_len + 16;
    const uint64_t stage_need = pk_off + (r.locked ? 0 : J.packets_len);
    const uint64_t res_need = verify ? n : 64 * n;
    if (dev_need > V.dev_ring.capacity() || stage_need > V.stage_ring.capacity() ||
        res_need > V.res_ring.capacity() || nchunks > V.chunks.capacity())
        return -1;
    if (V.free_slots.empty()) return 0;
    if (V.in_use + r.bytes > sv->cap && !V.inflight.empty()) return 0;   // wait for memory
    uint64_t dv, di, sp, si, rv, ri, cv, ci;
    if (!V.dev_ring.alloc(dev_need, 256, &dv, &di)) return 0;
    if (!V.stage_ring.alloc(stage_need, 256, &sp, &si)) {
        V.dev_ring.release(di);
        return 0;
    }
    if (!V.res_ring.alloc(res_need, 64, &rv, &ri)) {
        V.dev_ring.release(di);
        V.stage_ring.release(si);
        return 0;
    }
    if (!V.chunks.alloc(nchunks, 1, &cv, &ci)) {
        V.dev_ring.release(di);
        V.stage_ring.release(si);
        V.res_ring.release(ri);
        return 0;
    }
    const uint32_t slot = V.free_slots.back();
    V.free_slots.pop_back();
    uint32_t gen = V.gen[slot] + 1;
    if (gen == 0) gen = 1;
    V.gen[slot] = gen;
    uint8_t* stage = V.h_stage + sp % V.stage_ring.capacity();
    uint8_t* din = V.d_in + dv % V.dev_ring.capacity();
    uint8_t* res = V.h_res + rv % V.res_ring.capacity();
    // the job's own arrays, verbatim: each item's offsets are checked on the
    // GPU against the job's packet bytes
    uint32_t* hidx = reinterpret_cast<uint32_t*>(stage);
    memcpy(hidx, J.message_lens, 4 * n);
    memcpy(hidx + n, J.public_key_offsets, 4 * n);
    memcpy(hidx + 2 * n, J.key_offsets, 4 * n);
    memcpy(hidx + 3 * n, J.message_start_offsets, 4 * n);
    cudaError_t e = cudaSuccess;
    if (!r.locked && J.packets_len) {
        gb300::CopyPiece pc{stage + pk_off, J.packets, J.packets_len};
        gb300::CopyPool::copy(&pc, 1);
        e = cudaMemcpyAsync(din, stage, pk_off + J.packets_len, cudaMemcpyHostToDevice, V.copy);
    } else {
        e = cudaMemcpyAsync(din, stage, idx_bytes, cudaMemcpyHostToDevice, V.copy);
        if (e == cudaSuccess && J.packets_len)
            e = cudaMemcpyAsync(din + pk_off, J.packets, J.packets_len, cudaMemcpyHostToDevice, V.copy);
    }
    SvcReq& q = V.h_req[slot];
    const uint32_t* di32 = reinterpret_cast<const uint32_t*>(din);
    q.b = SigBatch{din + pk_off, J.packets_len, di32, di32 + n, di32 + 2 * n, di32 + 3 * n, (uint32_t)n,
                   V.d_res + rv % V.res_ring.capacity(), sv->info.tables};
    q.b.window = sv->info.verify_window;
    q.gen = gen;
    const uint32_t mode = verify ? (quad ? kSvcVerifyQuad : kSvcVerify) : kSvcSign;
    for (uint64_t k = 0; k < nchunks; k++) {
        SvcChunk& c = V.h_ring[(cv + k) % kSvcRing];
        c.req = slot;
        c.first = (uint32_t)(k * per);
        c.count = (uint32_t)std::min<uint64_t>(per, n - k * per);
        c.mode = mode;
    }
    V.chunk_tail = cv + nchunks;
    if (e == cudaSuccess) e = svc_publish(V, (uint32_t)V.chunk_tail);
    if (e != cudaSuccess) V.err = e;
    V.inflight.push_back({r.ticket, r.kind, slot, gen, n, J.out, res_need, res, di, si, ri, ci, r.bytes, now_ns()});
    V.in_use += r.bytes;
    V.max_inflight = std::max<uint64_t>(V.max_inflight, V.inflight.size());
    svc_ensure_running(sv);
    return 1;
}

// Completed requests out of the FIFO (results to the callers, ring space
// back), then queued requests in, then the kernel kept running (V.mu held).
void svc_progress(gb300_server* sv, std::vector<SvcDone>& done, std::vector<Req>& to_slots) {
    SigService& V = sv->svc;
    for (size_t k = 0; k < V.inflight.size();) {
        SvcInflight& f = V.inflight[k];
        const bool ok = __atomic_load_n(&V.h_done[f.slot], __ATOMIC_ACQUIRE) == f.gen;
        if (!ok && V.err == cudaSuccess) {
            k++;
            continue;
        }
        if (ok) memcpy(f.out, f.res, f.out_bytes);
        else memset(f.out, 0, f.out_bytes);
        float wait_ms = -1.f, run_ms = -1.f;
        if (ok) {
            const int64_t first = (int64_t)V.h_times[2 * f.slot] + V.clock_offset;
            const int64_t end = (int64_t)V.h_times[2 * f.slot + 1] + V.clock_offset;
            wait_ms = (float)((first - f.t_pub) * 1e-6);
            run_ms = (float)((end - first) * 1e-6);
        }
        done.push_back({f.ticket, f.n, ok ? 1 : -(int)V.err, f.t_pub, now_ns(), wait_ms, run_ms});
        V.dev_ring.release(f.id_dev);
        V.stage_ring.release(f.id_stage);
        V.res_ring.release(f.id_res);
        V.chunks.release(f.id_chunk);
        V.free_slots.push_back(f.slot);
        V.in_use -= f.dev_bytes;
        V.served++;
        f = V.inflight.back();
        V.inflight.pop_back();
    }
    while (!V.pending.empty()) {
        const int rc = svc_try_submit(sv, V.pending.front());
        if (rc == 0) break;
        if (rc < 0) {
            to_slots.push_back(V.pending.front());
            V.fallback++;
        }
        V.pending.pop_front();
    }
    svc_ensure_running(sv);
}

void dispatcher(gb300_server* sv) {
    cudaSetDevice(sv->dev);
    // the short waits below (a few us while the GPU has requests) would
    // otherwise overshoot by the default 50 us timer slack
    prctl(PR_SET_TIMERSLACK, 1000UL, 0, 0, 0);
    std::unique_lock<std::mutex> lk(sv->mu);
    std::vector<SvcDone> svc_done;
    std::vector<Req> to_slots;
    for (;;) {
        // ---- resident signature service: completions, queued requests ----
        bool svc_busy = false;
        if (sv->svc.on) {
            lk.unlock();
            {
                std::lock_guard<std::mutex> vl(sv->svc.mu);
                svc_progress(sv, svc_done, to_slots);
                svc_busy = !sv->svc.inflight.empty() || !sv->svc.pending.empty();
            }
            lk.lock();
            for (const SvcDone& d : svc_done) {
                auto it = sv->times.find(d.ticket);
                if (it != sv->times.end()) {
                    it->second.second = d.t_done;
                    if (sv->trace.size() >= kTraceCap) sv->trace.erase(sv->trace.begin(), sv->trace.begin() + kTraceCap / 4);
                    sv->trace.push_back({4, 1u, d.n, it->second.first, d.t_pub, d.t_done, d.wait_ms, d.run_ms,
                                         (float)((d.t_done - d.t_pub) * 1e-6)});
                }
                sv->status[d.ticket] = d.status;
                sv->requests_done++;
                sv->items_done += d.n;
            }
            if (!svc_done.empty()) sv->cv_done.notify_all();
            svc_done.clear();
            for (Req& r : to_slots) sv->pending_sig.push_back(r);
            to_slots.clear();
            if (sv->svc.max_inflight > sv->merged_max) sv->merged_max = sv->svc.max_inflight;
        }
        // ---- completions ----
        bool any_busy = false;
        for (auto* slots : {&sv->sig_slots, &sv->poh_slots}) {
            for (auto& S : *slots) {
                if (!S.busy) continue;
                cudaError_t q = S.err != cudaSuccess ? cudaSuccess : cudaEventQuery(S.done);
                if (q == cudaErrorNotReady) {
                    any_busy = true;
                    continue;
                }
                if (q != cudaSuccess && S.err == cudaSuccess) S.err = q;
                lk.unlock();
                // a launch that failed part-way may still have copies queued:
                // drain the stream before the slot's buffers are reused
                cudaStreamSynchronize(S.stream);
                cudaGetLastError();
                deliver(S);
                lk.lock();
                const int64_t t_done = now_ns();
                {
                    uint64_t it = 0;
                    for (auto& r : S.reqs) it += r.n;
                    if (sv->trace.size() >= kTraceCap) sv->trace.erase(sv->trace.begin(), sv->trace.begin() + kTraceCap / 4);
                    float ms_in = -1.f, ms_run = -1.f, ms_out = -1.f;
                    if (S.err == cudaSuccess) {
                        if (cudaEventElapsedTime(&ms_in, S.ev_in, S.ev_run) != cudaSuccess) ms_in = -1.f;
                        if (cudaEventElapsedTime(&ms_run, S.ev_run, S.ev_out) != cudaSuccess) ms_run = -1.f;
                        if (cudaEventElapsedTime(&ms_out, S.ev_out, S.done) != cudaSuccess) ms_out = -1.f;
                        cudaGetLastError();
                    }
                    sv->trace.push_back({S.kind, (uint32_t)S.reqs.size(), it, S.t_admit, S.t_enqueued, t_done, ms_in,
                                         ms_run, ms_out});
                }
                for (auto& r : S.reqs) {
                    sv->times[r.ticket].second = t_done;
                    sv->status[r.ticket] = S.err == cudaSuccess ? 1 : -(int)S.err;
                    sv->requests_done++;
                    sv->items_done += r.n;
                }
                sv->in_use -= S.bytes;
                S.reqs.clear();
                S.bytes = 0;
                S.busy = false;
                S.err = cudaSuccess;
                sv->cv_done.notify_all();
            }
        }
        // ---- admission ----
        bool launched = false;
        for (auto& S : sv->sig_slots) {
            if (S.busy || sv->pending_sig.empty()) continue;
            uint64_t items = 0, bytes = 0, pkt = 0;
            const bool wire = sv->pending_sig.front().kind == 3;
            const uint32_t stride = sv->pending_sig.front().stride;
            while (!sv->pending_sig.empty()) {
                const Req& r = sv->pending_sig.front();
                // merge while the launch fits the item cap, the memory budget
                // and the slot's resident packet ring (no reallocation; and
                // below 4 GiB, the reach of 32-bit packet offsets, should a
                // large request have grown the ring); one launch holds wire
                // packets of one stride or offset jobs
                const uint64_t ring = S.d_data.cap < 0xfffffff0ull ? S.d_data.cap : 0xfffffff0ull;
                if (!S.reqs.empty() && ((r.kind == 3) != wire || (wire && r.stride != stride) ||
                                        items + r.n > sv->max_items || sv->in_use + bytes + r.bytes > sv->cap ||
                                        pkt + r.ring_bytes + 16 > ring))
                    break;
                if (S.reqs.empty() && sv->in_use + r.bytes > sv->cap) break;   // wait for memory
                items += r.n;
                bytes += r.bytes;
                pkt += r.ring_bytes;
                S.reqs.push_back(r);
                sv->pending_sig.pop_front();
            }
            if (S.reqs.empty()) continue;
            S.busy = true;
            S.kind = wire ? 3 : 0;
            S.bytes = bytes;
            sv->in_use += bytes;
            sv->launches_sig++;
            if (S.reqs.size() > sv->merged_max) sv->merged_max = S.reqs.size();
            S.t_admit = now_ns();
            lk.unlock();
            S.err = wire ? launch_packets(sv, S) : launch_sigs(sv, S);
            S.t_enqueued = now_ns();
            lk.lock();
            launched = true;
        }
        for (auto& S : sv->poh_slots) {
            if (S.busy || sv->pending_poh.empty()) continue;
            uint64_t bytes = 0;
            while (!sv->pending_poh.empty()) {
                const Req& r = sv->pending_poh.front();
                if (sv->in_use + bytes + r.bytes > sv->cap) break;
                bytes += r.bytes;
                S.reqs.push_back(r);
                sv->pending_poh.pop_front();
            }
            if (S.reqs.empty()) continue;
            S.busy = true;
            S.kind = 2;
            S.bytes = bytes;
            sv->in_use += bytes;
            sv->launches_poh++;
            S.t_admit = now_ns();
            lk.unlock();
            S.err = launch_pohs(sv, S);
            S.t_enqueued = now_ns();
            lk.lock();
            launched = true;
        }
        if (launched) continue;
        bool busy = false;
        for (auto* slots : {&sv->sig_slots, &sv->poh_slots})
            for (auto& S : *slots) busy |= S.busy;
        if (sv->stop && !busy && !svc_busy && sv->pending_sig.empty() && sv->pending_poh.empty()) break;
        if (svc_busy)
            sv->cv_work.wait_for(lk, std::chrono::microseconds(5));
        else if (busy || any_busy)
            sv->cv_work.wait_for(lk, std::chrono::microseconds(20));
        else
            sv->cv_work.wait(lk);
    }
}

}  // namespace

extern "C" {

gb300_server* gb300_server_create(const gb300_server_config* cfg) {
    // more streams than hardware work queues would make signature launches
    // wait behind PoH kernels (see crypt_api.cu request_connections)
    if (!getenv("CUDA_DEVICE_MAX_CONNECTIONS")) setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    auto* sv = new gb300_server();
    sv->dev = dev;
    if (!crypt_device_info(dev, &sv->info)) {
        delete sv;
        return nullptr;
    }
    // PoH launches: paired warps, one pair per SM at most (2 x SMs warps).
    // Measured on GB300 under the served request mix, against independent
    // warps packed four to a block and against a pair on every other
    // sub-partition: the same signature peak (~8,950 requests/s) as the
    // packed warps with PoH latency p50 1.31 s instead of 1.86 s; two pairs
    // per SM cut the signature peak to ~7,300.  GB300_CRYPT_SERVER_POH_FORM
    // (a PohBatchForm) and GB300_CRYPT_SERVER_POH_WARPS override the shape.
    sv->poh_form = kPohPair;
    sv->poh_warps = sv->info.poh_warps / 2 > 2 ? sv->info.poh_warps / 2 : 2;
    if (const char* v = getenv("GB300_CRYPT_SERVER_POH_FORM")) {
        const int f = atoi(v);
        if (f >= kPohSingle && f <= kPohPackedPair) sv->poh_form = f;
    }
    if (const char* v = getenv("GB300_CRYPT_SERVER_POH_WARPS")) {
        const int w = atoi(v);
        if (w > 0 && w <= 64 * sv->info.sms) sv->poh_warps = w;
    }
    sv->cap = cfg && cfg->device_memory_cap ? cfg->device_memory_cap : (8ull << 30);
    sv->max_items = cfg && cfg->max_items_per_launch ? cfg->max_items_per_launch : 65536u;
    const bool service = !cfg || cfg->sig_mode == 0;
    // with the service, slots carry only wire-packet batches and jobs too
    // large for the service's rings
    const uint32_t nsig = cfg && cfg->sig_slots ? cfg->sig_slots : (service ? 2u : 3u);
    const uint32_t npoh = cfg && cfg->poh_slots ? cfg->poh_slots : 2u;
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);   // hi is the numerically smaller, higher priority
    sv->sig_slots.resize(nsig);
    sv->poh_slots.resize(npoh);
    bool ok = true;
    for (auto& S : sv->sig_slots)
        ok = ok && cudaStreamCreateWithPriority(&S.stream, cudaStreamNonBlocking, hi) == cudaSuccess &&
             cudaEventCreate(&S.done) == cudaSuccess && cudaEventCreate(&S.ev_in) == cudaSuccess &&
             cudaEventCreate(&S.ev_run) == cudaSuccess && cudaEventCreate(&S.ev_out) == cudaSuccess;
    for (auto& S : sv->poh_slots)
        ok = ok && cudaStreamCreateWithPriority(&S.stream, cudaStreamNonBlocking, lo) == cudaSuccess &&
             cudaEventCreate(&S.done) == cudaSuccess && cudaEventCreate(&S.ev_in) == cudaSuccess &&
             cudaEventCreate(&S.ev_run) == cudaSuccess && cudaEventCreate(&S.ev_out) == cudaSuccess;
    // resident rings: each signature slot holds a 64 MiB packet ring and the
    // index/output space of a full launch; each PoH slot 65536 entries
    for (auto& S : sv->sig_slots) {
        const uint64_t mi = sv->max_items;
        ok = ok && S.d_data.ensure(64ull << 20, S.stream) == cudaSuccess &&
             S.d_index.ensure(16 * mi, S.stream) == cudaSuccess &&
             S.d_out.ensure(round_up(mi, 64) + 64 * mi, S.stream) == cudaSuccess &&
             S.d_scratch.ensure(256, S.stream) == cudaSuccess &&
             S.h_stage.ensure(round_up(16 * mi, 256) + (64ull << 20)) == cudaSuccess &&
             S.h_out.ensure(round_up(mi, 64) + 64 * mi) == cudaSuccess;
    }
    for (auto& S : sv->poh_slots) {
        ok = ok && S.d_data.ensure(40ull * 65536, S.stream) == cudaSuccess &&
             S.d_scratch.ensure(poh_batch_workspace_size(65536), S.stream) == cudaSuccess &&
             S.h_stage.ensure(40ull * 65536) == cudaSuccess;
    }
    for (auto* slots : {&sv->sig_slots, &sv->poh_slots})
        for (auto& S : *slots) ok = ok && cudaStreamSynchronize(S.stream) == cudaSuccess;
    if (ok && service) ok = svc_create(sv);
    if (!ok) {
        gb300_server_destroy(sv);
        return nullptr;
    }
    sv->worker = std::thread(dispatcher, sv);
    return sv;
}

void gb300_server_destroy(gb300_server* sv) {
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(sv->dev);
    // PoH launches read the service's FIFO words (PohYield): every slot's
    // work ends before the service state is freed
    for (auto* slots : {&sv->sig_slots, &sv->poh_slots})
        for (auto& S : *slots)
            if (S.stream) cudaStreamSynchronize(S.stream);
    svc_destroy(sv);
    for (auto* slots : {&sv->sig_slots, &sv->poh_slots})
        for (auto& S : *slots) {
            S.d_data.release();
            S.d_index.release();
            S.d_out.release();
            S.d_scratch.release();
            S.h_stage.release();
            S.h_out.release();
            for (cudaEvent_t ev : {S.done, S.ev_in, S.ev_run, S.ev_out})
                if (ev) cudaEventDestroy(ev);
            if (S.stream) cudaStreamDestroy(S.stream);
        }
    if (prev >= 0) cudaSetDevice(prev);
    delete sv;
}

uint64_t gb300_server_submit_sigs(gb300_server* sv, const gb300_sig_job* job) {
    if (!sv || !job || job->kind > 1 || job->num == 0 || !job->out || !job->message_lens ||
        !job->public_key_offsets || !job->key_offsets || !job->message_start_offsets ||
        (job->packets_len && !job->packets) || job->packets_len >= 0xfffffff0ull)
        return 0;
    Req r;
    r.kind = (int)job->kind;
    r.job = *job;
    r.n = job->num;
    r.ring_bytes = job->packets_len;
    r.locked = !job->packets_len || page_locked(job->packets);
    r.bytes = sig_bytes(*job);
    if (r.bytes > sv->cap) return 0;   // a request above max_items runs in a launch of its own
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        r.ticket = sv->next_ticket++;
        sv->status[r.ticket] = 0;
        sv->times[r.ticket] = {now_ns(), -1};
    }
    if (sv->svc.on) {
        // staged and published from this thread, in arrival order
        int rc = 0;
        {
            std::lock_guard<std::mutex> vl(sv->svc.mu);
            rc = sv->svc.pending.empty() ? svc_try_submit(sv, r) : 0;
            if (rc == 0) sv->svc.pending.push_back(r);
            if (rc < 0) sv->svc.fallback++;
        }
        if (rc >= 0) {
            sv->cv_work.notify_one();
            return r.ticket;
        }
    }
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->pending_sig.push_back(r);
    sv->cv_work.notify_one();
    return r.ticket;
}

uint64_t gb300_server_submit_packets(gb300_server* sv, const gpu_Elems* elems, uint32_t num_elems, uint32_t stride,
                                     const uint32_t* packet_lens, uint8_t* packet_out, uint32_t* sig_counts) {
    if (!sv || !elems || num_elems == 0 || stride == 0 || !packet_lens || !packet_out) return 0;
    Req r;
    r.kind = 3;
    r.stride = stride;
    r.lens = packet_lens;
    r.pkt_out = packet_out;
    r.sig_counts = sig_counts;
    for (uint32_t i = 0; i < num_elems; i++) {
        if (elems[i].num && !elems[i].elems) return 0;
        r.n += elems[i].num;
    }
    // packet offsets are 32-bit, as in the one-call form
    if (r.n == 0 || r.n * stride > 0xffffffffull) return 0;
    r.elems.assign(elems, elems + num_elems);
    r.locked = true;
    for (const gpu_Elems& g : r.elems)
        if (g.num && r.locked) r.locked = page_locked(g.elems);
    r.ring_bytes = r.n * stride;
    r.bytes = r.ring_bytes + 4 * r.n + pkt_counts_off(r.n) + 4 * r.n +
              packets_workspace_size((uint32_t)r.n, stride) + 64;
    if (r.bytes > sv->cap) return 0;
    std::lock_guard<std::mutex> lk(sv->mu);
    const uint64_t t = r.ticket = sv->next_ticket++;
    sv->status[t] = 0;
    sv->times[t] = {now_ns(), -1};
    sv->pending_sig.push_back(std::move(r));
    sv->cv_work.notify_one();
    return t;
}

uint64_t gb300_server_submit_poh(gb300_server* sv, uint8_t* hashes, const uint64_t* num_hashes, size_t num_elems) {
    if (!sv || !hashes || !num_hashes || num_elems == 0 || num_elems > 0x7fffffffull) return 0;
    Req r;
    r.kind = 2;
    r.hashes = hashes;
    r.counts = num_hashes;
    r.n = num_elems;
    r.bytes = 40ull * num_elems + poh_batch_workspace_size(num_elems);
    if (r.bytes > sv->cap) return 0;
    std::lock_guard<std::mutex> lk(sv->mu);
    r.ticket = sv->next_ticket++;
    sv->status[r.ticket] = 0;
    sv->times[r.ticket] = {now_ns(), -1};
    sv->pending_poh.push_back(r);
    sv->cv_work.notify_one();
    return r.ticket;
}

int gb300_server_poll(gb300_server* sv, uint64_t ticket) {
    if (!sv) return -(int)cudaErrorInvalidValue;
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->status.find(ticket);
    return it == sv->status.end() ? -(int)cudaErrorInvalidValue : it->second;
}

int gb300_server_wait(gb300_server* sv, uint64_t ticket, int timeout_ms) {
    if (!sv) return -(int)cudaErrorInvalidValue;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto done = [&]() {
        auto it = sv->status.find(ticket);
        return it == sv->status.end() || it->second != 0;
    };
    if (timeout_ms < 0)
        sv->cv_done.wait(lk, done);
    else
        sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done);
    auto it = sv->status.find(ticket);
    return it == sv->status.end() ? -(int)cudaErrorInvalidValue : it->second;
}

void gb300_server_release(gb300_server* sv, uint64_t ticket) {
    if (!sv) return;
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->status.find(ticket);
    if (it != sv->status.end() && it->second != 0) {
        sv->status.erase(it);
        sv->times.erase(ticket);
    }
}

int gb300_server_times(gb300_server* sv, uint64_t ticket, int64_t* submit_ns, int64_t* done_ns) {
    if (!sv) return -(int)cudaErrorInvalidValue;
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->times.find(ticket);
    if (it == sv->times.end()) return -(int)cudaErrorInvalidValue;
    if (submit_ns) *submit_ns = it->second.first;
    if (done_ns) *done_ns = it->second.second;
    return it->second.second >= 0 ? 1 : 0;
}

int gb300_server_trace(gb300_server* sv, char* buf, size_t len) {
    if (!sv || !buf || len == 0) return 0;
    std::lock_guard<std::mutex> lk(sv->mu);
    size_t off = 0;
    int n = snprintf(buf, len, "[");
    if (n < 0) return 0;
    off = (size_t)n;
    for (size_t i = 0; i < sv->trace.size() && off + 128 < len; i++) {
        const auto& t = sv->trace[i];
        n = snprintf(buf + off, len - off, "%s[%d,%u,%llu,%lld,%lld,%lld,%.4f,%.4f,%.4f]", i ? "," : "", t.kind,
                     t.reqs, (unsigned long long)t.items, (long long)t.t_admit, (long long)t.t_enqueued,
                     (long long)t.t_complete, t.copy_in_ms, t.kernels_ms, t.copy_out_ms);
        if (n < 0) break;
        off += (size_t)n;
    }
    if (off + 2 <= len) {
        buf[off++] = ']';
        buf[off] = 0;
    }
    return (int)off;
}

int gb300_server_stats(gb300_server* sv, char* buf, size_t len) {
    if (!sv || !buf || len == 0) return 0;
    std::lock_guard<std::mutex> lk(sv->mu);
    uint64_t sl = 0, sm = 0, ss = 0, sf = 0, sp = 0, si = 0;
    {
        std::lock_guard<std::mutex> vl(sv->svc.mu);
        sl = sv->svc.launches;
        sm = sv->svc.max_inflight;
        ss = sv->svc.served;
        sf = sv->svc.fallback;
        sp = sv->svc.pending.size();
        si = sv->svc.in_use;
    }
    int n = snprintf(buf, len,
                     "{\"device\": %d, \"launches_sig\": %llu, \"launches_poh\": %llu, \"requests_done\": %llu, "
                     "\"items_done\": %llu, \"max_requests_merged\": %llu, \"pending_sig\": %zu, "
                     "\"pending_poh\": %zu, \"device_bytes_in_flight\": %llu, \"device_memory_cap\": %llu, "
                     "\"service\": {\"on\": %d, \"launches\": %llu, \"max_in_flight\": %llu, \"served\": %llu, "
                     "\"to_slots\": %llu, \"pending\": %llu, \"device_bytes_in_flight\": %llu}}",
                     sv->dev, (unsigned long long)(sv->launches_sig + sl), (unsigned long long)sv->launches_poh,
                     (unsigned long long)sv->requests_done, (unsigned long long)sv->items_done,
                     (unsigned long long)sv->merged_max, sv->pending_sig.size(), sv->pending_poh.size(),
                     (unsigned long long)sv->in_use, (unsigned long long)sv->cap, sv->svc.on ? 1 : 0,
                     (unsigned long long)sl, (unsigned long long)sm, (unsigned long long)ss, (unsigned long long)sf,
                     (unsigned long long)sp, (unsigned long long)si);
    return n < 0 ? 0 : (n < (int)len ? n : (int)len - 1);
}

}  // extern "C"
