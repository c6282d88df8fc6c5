// C ABI of libcuda-crypt.so: the reference's entry points (include/ed25519.h,
// include/poh_verify.h) over a pool of GPU queues.
//
// Replaces the reference's host drivers and context pool
// (src/cuda-ecc-ed25519/gpu_ctx.cu:8-165, verify.cu:240-340,
// sign.cu:76-145, src/cuda-poh-verify/poh_verify.cu:29-144).
// Same pool shape (up to 8 GPUs x 8 queues, one lock per queue, grow-only
// device buffers) shared by every entry point; calls go round-robin over
// the GPUs as in the reference, but within a GPU to its first idle queue
// rather than the next one, so that a lone caller keeps reusing one queue's
// buffers and captured graphs.  In addition:
//   * a grow-only page-locked staging buffer per queue: the four per-
//     signature index arrays and the packets go to the GPU in one copy
//     (packets that the caller page-locked with cuda_host_register are
//     copied straight from the caller's memory instead);
//   * argument checks and error codes instead of assert() aborts;
//   * device tables (curve constants, basepoint multiples) built on the GPU
//     when the pool is created.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "ed25519.h"
#include "poh_verify.h"
#include "gb300_packets.h"
#include "gb300_diag.h"
#include "kernels.h"
#include "tables.cuh"
#include "host_buffers.h"
#include "host_copy.h"
#include "queue_pick.h"

#include <functional>

namespace {

using gb300::DevBuf;
using gb300::HostBuf;
using gb300::round_up;

constexpr int kMaxGpus = 8;
constexpr int kQueues = 8;

std::atomic<bool> g_verbose{false};
thread_local int t_last_error = 0;

#define LOG(...)                                       \
    do {                                               \
        if (g_verbose.load(std::memory_order_relaxed)) { \
            printf(__VA_ARGS__);                       \
            fflush(stdout);                            \
        }                                              \
    } while (0)

// A captured launch sequence, replayed while its key (sizes, buffer
// addresses, launch shape) stays the same.
struct GraphCache {
    cudaGraphExec_t exec = nullptr;
    std::vector<uint64_t> key;
    void reset() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        key.clear();
    }
};

struct Queue {
    std::mutex mu;
    cudaStream_t stream = nullptr;
    DevBuf d_data, d_index, d_out, d_scratch;
    HostBuf h_stage, h_out;
    GraphCache g_poh, g_sig, g_pkt;
    void release_buffers() {
        g_poh.reset();
        g_sig.reset();
        g_pkt.reset();
        d_data.release();
        d_index.release();
        d_out.release();
        d_scratch.release();
        h_stage.release();
        h_out.release();
    }
};

// Launch shapes picked by the autotuner (tune_device) for one GPU.
struct Tuning {
    int sig_threads = 128;        // threads per block of the persistent sign/verify kernel
    int sig_blocks_per_sm = 0;    // 0 = as many as fit
    int verify_window = 0;        // one-lane verify: 0 half-size scalars, or the window width of h (4 or 5)
    int poh_warps_per_smsp = 1;   // resident warps of the persistent PoH kernel per SM sub-partition
    int poh_form = kPohSingle;    // PohBatchForm of ragged PoH batches
    double sig_ms[2][3] = {{0, 0, 0}, {0, 0, 0}};  // calibration: half-size scalars / window 4 x 64 / 128 / 256 threads
    double poh_ms[4] = {0, 0, 0, 0};  // calibration: single and paired forms, 1 and 2 warps per sub-partition
    int calib_sigs = 0, calib_chains = 0;
};

struct Device {
    int id = -1;
    int sms = 0;
    CurveTables* tables = nullptr;
    Queue q[kQueues];
    std::once_flag tuned;
    std::atomic<bool> tuned_done{false};
    Tuning tune;
};

std::mutex g_mu;
int g_num_gpus = -1;  // -1: not initialised yet
Device g_dev[kMaxGpus];
gb300::QueueTurns<kMaxGpus> g_turns;     // round-robin state, under g_mu

// Streams beyond CUDA_DEVICE_MAX_CONNECTIONS (default 8) share hardware work
// queues, so a short verify launch can end up queued behind a second-long
// PoH kernel on an unrelated stream.  Ask for the maximum before the CUDA
// context exists (it has no effect once the process has created it; a host
// application that creates it first should set the variable itself).
void request_connections() {
    if (!getenv("CUDA_DEVICE_MAX_CONNECTIONS")) setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
}

bool init_locked() {
    if (g_num_gpus >= 0) return g_num_gpus > 0;
    request_connections();
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    if (n > kMaxGpus) n = kMaxGpus;
    int prev = -1;
    cudaGetDevice(&prev);
    int usable = 0;
    for (int d = 0; d < n; d++) {
        if (cudaSetDevice(d) != cudaSuccess) break;
        Device& D = g_dev[d];
        D.id = d;
        // queue 0's stream now (tables); the others on first use
        bool ok = cudaStreamCreateWithFlags(&D.q[0].stream, cudaStreamNonBlocking) == cudaSuccess;
        if (ok) ok = crypt_tables_create(&D.tables, D.q[0].stream) == cudaSuccess;
        if (ok) ok = cudaDeviceGetAttribute(&D.sms, cudaDevAttrMultiProcessorCount, d) == cudaSuccess;
        // every kernel of the library loaded now, not at its first launch
        // (which may then wait for running kernels: see load_kernels)
        if (ok)
            ok = preload_verify_kernels() == cudaSuccess && preload_sign_kernels() == cudaSuccess &&
                 preload_poh_kernels() == cudaSuccess && preload_poh_batch_kernels() == cudaSuccess &&
                 preload_sig_batch_kernels() == cudaSuccess && preload_packets_kernels() == cudaSuccess &&
                 preload_sig_service_kernels() == cudaSuccess && preload_poh_entries_kernels() == cudaSuccess;
        if (!ok) {
            fprintf(stderr, "libcuda-crypt: GPU %d unusable: %s\n", d, cudaGetErrorString(cudaGetLastError()));
            break;
        }
        usable = d + 1;
    }
    if (prev >= 0) cudaSetDevice(prev);
    g_num_gpus = usable;
    LOG("total_gpus: %d\n", usable);
    return usable > 0;
}

struct Lease {
    Device* dev = nullptr;
    Queue* q = nullptr;
    ~Lease() {
        if (q) q->mu.unlock();
    }
};

// GPU round-robin, then the GPU's first idle queue (the next one in turn
// when all are busy), then the queue's lock: gb300::pick_queue
// (queue_pick.h).  The reference (gpu_ctx.cu:46-73) picks the next queue in
// turn every time: a caller issuing one call after another then meets every
// queue's first-use buffer growth and graph capture; measured on GB300 for
// 131 MB ragged batches: 15.4 ms per call in turn against 9.2 ms on the
// warm queue.
bool acquire(Lease& L) {
    std::unique_lock<std::mutex> lk(g_mu);
    if (!init_locked()) return false;
    const gb300::QueuePick p = gb300::pick_queue(
        g_turns, g_num_gpus, kQueues, [](int g, int k) { return g_dev[g].q[k].mu.try_lock(); });
    lk.unlock();
    Device& D = g_dev[p.gpu];
    Queue& Q = D.q[p.queue];
    if (!p.held) Q.mu.lock();
    L.dev = &D;
    L.q = &Q;
    cudaSetDevice(D.id);
    if (!Q.stream && cudaStreamCreateWithFlags(&Q.stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        Q.mu.unlock();
        L.q = nullptr;
        return false;
    }
    return true;
}

const CurveTables* tables_for_current_device() {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!init_locked() || dev < 0 || dev >= g_num_gpus) return nullptr;
    return g_dev[dev].tables;
}

bool is_page_locked(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

#define TRY(expr)                                   \
    do {                                            \
        cudaError_t _e = (expr);                    \
        if (_e != cudaSuccess) return _e;           \
    } while (0)


// GB300_CRYPT_NO_GRAPH=1 enqueues the launches directly instead.
template <class F>
cudaError_t run_graph(GraphCache& gc, const std::vector<uint64_t>& key, cudaStream_t s, F&& enqueue) {
    static const bool no_graph = getenv("GB300_CRYPT_NO_GRAPH") && atoi(getenv("GB300_CRYPT_NO_GRAPH")) != 0;
    if (no_graph) return enqueue(s);
    if (gc.exec && gc.key == key) return cudaGraphLaunch(gc.exec, s);
    gc.reset();
    cudaGraph_t g = nullptr;
    TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue(s);
    cudaError_t e2 = cudaStreamEndCapture(s, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return e != cudaSuccess ? e : e2;
    }
    e = cudaGraphInstantiate(&gc.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        gc.exec = nullptr;
        return e;
    }
    gc.key = key;
    return cudaGraphLaunch(gc.exec, s);
}

int env_int(const char* name, int dflt) {
    const char* v = getenv(name);
    return v && *v ? atoi(v) : dflt;
}

uint64_t splitmix(uint64_t& x) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

float time_ms(cudaStream_t s, const std::function<cudaError_t()>& f, cudaError_t& err) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
    err = f();
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms;
}

// Calibrates the persistent kernels on this GPU (about a few hundred ms,
// once per device): the sign/verify kernel on valid signatures it makes with
// its own keypair and sign kernels, the PoH kernel on ragged chains.
// GB300_CRYPT_SIG_THREADS / GB300_CRYPT_SIG_BLOCKS /
// GB300_CRYPT_POH_WARPS_PER_SMSP override the choices.
void tune_device(Device& D) {
    Tuning& T = D.tune;
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return;
    const int sms = D.sms > 0 ? D.sms : 1;
    // ---- signatures ----
    const uint32_t nv = (uint32_t)sms * 128u, ns = nv / 4u, stride = 224u;
    std::vector<uint8_t> hseed(32ull * nv), hpkt((size_t)stride * nv);
    std::vector<uint32_t> hidx(4ull * nv + 4ull * ns);
    uint64_t rs = 0x5eed;
    for (auto& b : hseed) b = (uint8_t)splitmix(rs);
    for (size_t i = 0; i < hpkt.size(); i++) hpkt[i] = (uint8_t)splitmix(rs);
    for (uint32_t i = 0; i < nv; i++) {
        hidx[i] = 64;                         // v lens
        hidx[nv + i] = stride * i + 64;       // v pk
        hidx[2 * nv + i] = stride * i;        // v sig
        hidx[3 * nv + i] = stride * i + 160;  // v msg
    }
    for (uint32_t i = 0; i < ns; i++) {
        hidx[4 * nv + i] = 64;
        hidx[4 * nv + ns + i] = stride * i + 64;
        hidx[4 * nv + 2 * ns + i] = stride * i + 96;   // sk
        hidx[4 * nv + 3 * ns + i] = stride * i + 160;
    }
    uint8_t *dseed = nullptr, *dpk = nullptr, *dsk = nullptr, *dsig = nullptr, *dpkt = nullptr, *dout = nullptr;
    uint32_t *didx = nullptr, *dq = nullptr;
    bool ok = cudaMalloc(&dseed, 32ull * nv) == cudaSuccess && cudaMalloc(&dpk, 32ull * nv) == cudaSuccess &&
              cudaMalloc(&dsk, 64ull * nv) == cudaSuccess && cudaMalloc(&dsig, 64ull * nv) == cudaSuccess &&
              cudaMalloc(&dpkt, hpkt.size()) == cudaSuccess && cudaMalloc(&dout, round_up(nv, 64) + 64ull * ns) == cudaSuccess &&
              cudaMalloc(&didx, 4ull * hidx.size()) == cudaSuccess && cudaMalloc(&dq, 16) == cudaSuccess;
    if (ok) {
        cudaMemcpyAsync(dseed, hseed.data(), hseed.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dpkt, hpkt.data(), hpkt.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(didx, hidx.data(), 4ull * hidx.size(), cudaMemcpyHostToDevice, s);
        launch_ed25519_keypair(dseed, dpk, dsk, nv, D.tables, s);
        cudaMemcpy2DAsync(dpkt + 64, stride, dpk, 32, 32, nv, cudaMemcpyDeviceToDevice, s);
        cudaMemcpy2DAsync(dpkt + 96, stride, dsk, 64, 64, nv, cudaMemcpyDeviceToDevice, s);
        SigBatch sb{dpkt, hpkt.size(), didx, didx + nv, nullptr, didx + 3 * nv, nv, dsig, D.tables};
        // sign every packet (private key at +96) to get valid signatures
        std::vector<uint32_t> skoff(nv);
        for (uint32_t i = 0; i < nv; i++) skoff[i] = stride * i + 96;
        uint32_t* dsko = nullptr;
        if (cudaMalloc(&dsko, 4ull * nv) == cudaSuccess) {
            cudaMemcpyAsync(dsko, skoff.data(), 4ull * nv, cudaMemcpyHostToDevice, s);
            sb.signature_offsets = dsko;
            launch_ed25519_sign(sb, s);
            cudaMemcpy2DAsync(dpkt, stride, dsig, 64, 64, nv, cudaMemcpyDeviceToDevice, s);
            cudaStreamSynchronize(s);
            cudaFree(dsko);
        }
        SigWork w;
        w.v = SigBatch{dpkt, hpkt.size(), didx, didx + nv, didx + 2 * nv, didx + 3 * nv, nv, dout, D.tables};
        w.s = SigBatch{dpkt, hpkt.size(), didx + 4 * nv, didx + 4 * nv + ns, didx + 4 * nv + 2 * ns,
                       didx + 4 * nv + 3 * ns, ns, dout + round_up(nv, 64), D.tables};
        w.sign_base = (nv + 31u) / 32u * 32u;
        w.total_chunks = (w.sign_base + ns + 31u) / 32u;
        w.next = dq;
        // the default (half-size scalars, 128 threads) is timed first;
        // another shape replaces it only when it is more than 2 % faster, so
        // timing noise does not move the choice from run to run
        const int cand[3] = {128, 64, 256};
        const int windows[2] = {0, 4};
        double best = 1e30;
        for (int wi = 0; wi < 2; wi++) {
            w.v.window = windows[wi];
            for (int c = 0; c < 3; c++) {
                cudaError_t err = cudaSuccess;
                launch_sig_batch(w, cand[c], 0, sms, s);   // warm
                cudaStreamSynchronize(s);
                float ms = 1e30f;
                for (int r = 0; r < 2; r++) {
                    float t = time_ms(s, [&]() { return launch_sig_batch(w, cand[c], 0, sms, s); }, err);
                    if (err == cudaSuccess && t < ms) ms = t;
                }
                T.sig_ms[wi][cand[c] == 64 ? 0 : cand[c] == 128 ? 1 : 2] = ms;
                if (best == 1e30 || ms < 0.98 * best) {
                    best = ms;
                    T.sig_threads = cand[c];
                    T.verify_window = windows[wi];
                }
            }
        }
        T.calib_sigs = (int)(nv + ns);
    }
    cudaFree(dseed); cudaFree(dpk); cudaFree(dsk); cudaFree(dsig); cudaFree(dpkt); cudaFree(dout); cudaFree(didx);
    // ---- PoH: ragged chains, counts log-uniform in 1..20000 (the longest
    // chain bounds the launch, as in real ragged batches) ----
    const uint32_t nc = 16384;
    std::vector<uint8_t> hh(32ull * nc);
    std::vector<uint64_t> hc(nc);
    for (auto& b : hh) b = (uint8_t)splitmix(rs);
    for (auto& c : hc) {
        const double u = (double)(splitmix(rs) >> 11) * (1.0 / 9007199254740992.0);
        c = (uint64_t)exp(u * log(20001.0));
        if (c < 1) c = 1;
        if (c > 20000) c = 20000;
    }
    uint8_t* dh = nullptr;
    uint64_t* dc = nullptr;
    void* ws = nullptr;
    if (cudaMalloc(&dh, hh.size()) == cudaSuccess && cudaMalloc(&dc, 8ull * nc) == cudaSuccess &&
        cudaMalloc(&ws, poh_batch_workspace_size(nc)) == cudaSuccess) {
        cudaMemcpyAsync(dh, hh.data(), hh.size(), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dc, hc.data(), 8ull * nc, cudaMemcpyHostToDevice, s);
        double best = 1e30;
        const int mode_wps[4] = {1, 2, 1, 2}, mode_form[4] = {kPohSingle, kPohSingle, kPohPair, kPohPair};
        for (int m = 0; m < 4; m++) {
            cudaError_t err = cudaSuccess;
            launch_poh_batch(dh, dc, nc, ws, 4 * sms * mode_wps[m], s, mode_form[m]);   // warm
            cudaStreamSynchronize(s);
            float ms = time_ms(
                s, [&]() { return launch_poh_batch(dh, dc, nc, ws, 4 * sms * mode_wps[m], s, mode_form[m]); }, err);
            T.poh_ms[m] = ms;
            if (err == cudaSuccess && ms < best) {
                best = ms;
                T.poh_warps_per_smsp = mode_wps[m];
                T.poh_form = mode_form[m];
            }
        }
        T.calib_chains = (int)nc;
    }
    cudaFree(dh); cudaFree(dc); cudaFree(ws); cudaFree(dq);
    cudaGetLastError();
    cudaStreamDestroy(s);
    T.sig_threads = env_int("GB300_CRYPT_SIG_THREADS", T.sig_threads);
    T.sig_blocks_per_sm = env_int("GB300_CRYPT_SIG_BLOCKS", T.sig_blocks_per_sm);
    {
        const int wv = env_int("GB300_CRYPT_VERIFY_WINDOW", T.verify_window);
        T.verify_window = (wv == 4 || wv == 5) ? wv : 0;
    }
    T.poh_warps_per_smsp = env_int("GB300_CRYPT_POH_WARPS_PER_SMSP", T.poh_warps_per_smsp);
    T.poh_form = env_int("GB300_CRYPT_POH_PAIRED", T.poh_form == kPohPair) ? kPohPair : kPohSingle;
    LOG("tuned gpu %d: sig threads %d window %d (ms %.3f %.3f %.3f / %.3f %.3f %.3f), poh warps/smsp %d %s "
        "(ms %.3f %.3f %.3f %.3f)\n", D.id, T.sig_threads, T.verify_window, T.sig_ms[0][0], T.sig_ms[0][1],
        T.sig_ms[0][2], T.sig_ms[1][0], T.sig_ms[1][1], T.sig_ms[1][2], T.poh_warps_per_smsp,
        T.poh_form == kPohPair ? "paired" : "single", T.poh_ms[0], T.poh_ms[1], T.poh_ms[2], T.poh_ms[3]);
}

Device* current_device() {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!init_locked() || dev < 0 || dev >= g_num_gpus) return nullptr;
    return &g_dev[dev];
}

const Tuning& tuning_for(Device& D) {
    std::call_once(D.tuned, [&]() {
        int prev = -1;
        cudaGetDevice(&prev);
        cudaSetDevice(D.id);
        tune_device(D);
        if (prev >= 0) cudaSetDevice(prev);
        D.tuned_done.store(true);
    });
    return D.tune;
}

// The tuned verify window when the device has been tuned, else 4: the
// one-call device entry points do not start the tuner (it allocates and
// synchronises, which a caller capturing a graph cannot allow).
int verify_window_if_tuned(Device& D) { return D.tuned_done.load() ? D.tune.verify_window : 0; }

// Stages one signature batch, runs verify or sign on it and copies the
// results into `out` (n bytes, or 64n bytes for signing).
cudaError_t run_sig_batch(Lease& L, cudaStream_t s, bool sign, const gpu_Elems* elems, uint32_t num_elems,
                          uint32_t message_size, uint64_t total_bytes, uint32_t n, const uint32_t* lens,
                          const uint32_t* key_offs, const uint32_t* sig_offs, const uint32_t* msg_offs,
                          uint8_t* out) {
    Queue& Q = *L.q;
    const size_t idx_bytes = 16ull * n;
    const size_t out_bytes = sign ? 64ull * n : (size_t)n;
    bool all_locked = true;
    for (uint32_t i = 0; i < num_elems && all_locked; i++)
        if (elems[i].num) all_locked = is_page_locked(elems[i].elems);
    const size_t stage_pk_off = round_up(idx_bytes, 256);
    const size_t stage_bytes = stage_pk_off + (all_locked ? 0 : total_bytes);

    TRY(Q.d_data.ensure(total_bytes + 16, s));
    TRY(Q.d_index.ensure(idx_bytes, s));
    TRY(Q.d_out.ensure(out_bytes, s));
    TRY(Q.h_stage.ensure(stage_bytes));
    TRY(Q.h_out.ensure(out_bytes));

    uint32_t* hidx = static_cast<uint32_t*>(Q.h_stage.p);
    memcpy(hidx, lens, 4ull * n);
    memcpy(hidx + n, key_offs, 4ull * n);
    memcpy(hidx + 2ull * n, sig_offs, 4ull * n);
    memcpy(hidx + 3ull * n, msg_offs, 4ull * n);
    TRY(cudaMemcpyAsync(Q.d_index.p, hidx, idx_bytes, cudaMemcpyHostToDevice, s));

    uint8_t* dpk = static_cast<uint8_t*>(Q.d_data.p);
    if (all_locked) {
        uint64_t cur = 0;
        for (uint32_t i = 0; i < num_elems; i++) {
            uint64_t b = (uint64_t)elems[i].num * message_size;
            if (b) TRY(cudaMemcpyAsync(dpk + cur, elems[i].elems, b, cudaMemcpyHostToDevice, s));
            cur += b;
        }
    } else {
        uint8_t* img = static_cast<uint8_t*>(Q.h_stage.p) + stage_pk_off;
        std::vector<gb300::CopyPiece> pcs;
        uint64_t cur = 0;
        for (uint32_t i = 0; i < num_elems; i++) {
            uint64_t b = (uint64_t)elems[i].num * message_size;
            if (b) pcs.push_back({img + cur, elems[i].elems, b});
            cur += b;
        }
        gb300::CopyPool::copy(pcs.data(), pcs.size());
        if (total_bytes) TRY(cudaMemcpyAsync(dpk, img, total_bytes, cudaMemcpyHostToDevice, s));
    }

    const uint32_t* didx = static_cast<const uint32_t*>(Q.d_index.p);
    SigBatch b;
    b.packets = dpk;
    b.packets_len = total_bytes;
    b.message_lens = didx;
    b.public_key_offsets = didx + n;
    b.signature_offsets = didx + 2ull * n;
    b.message_start_offsets = didx + 3ull * n;
    b.n = n;
    b.out = static_cast<uint8_t*>(Q.d_out.p);
    b.tables = L.dev->tables;
    b.window = tuning_for(*L.dev).verify_window;
    TRY(sign ? launch_ed25519_sign(b, s) : launch_ed25519_verify(b, s));
    TRY(cudaMemcpyAsync(Q.h_out.p, Q.d_out.p, out_bytes, cudaMemcpyDeviceToHost, s));
    TRY(cudaStreamSynchronize(s));
    memcpy(out, Q.h_out.p, out_bytes);
    return cudaSuccess;
}

void sig_many(bool sign, const gpu_Elems* elems, uint32_t num_elems, uint32_t message_size, uint32_t total_packets,
              uint32_t total_signatures, const uint32_t* message_lens, const uint32_t* key_offsets,
              const uint32_t* sig_offsets, const uint32_t* message_start_offsets, uint8_t* out,
              uint8_t use_non_default_stream) {
    LOG("Starting %s_many: num_elems: %u total_signatures: %u total_packets: %u message_size: %u\n",
        sign ? "sign" : "verify", num_elems, total_signatures, total_packets, message_size);
    if (total_packets == 0 || total_signatures == 0) return;
    const size_t out_bytes = sign ? 64ull * total_signatures : (size_t)total_signatures;
    if (!elems || !message_lens || !key_offsets || !sig_offsets || !message_start_offsets || !out) {
        t_last_error = cudaErrorInvalidValue;
        if (out) memset(out, 0, out_bytes);
        return;
    }
    uint64_t total_bytes = 0;
    for (uint32_t i = 0; i < num_elems; i++) total_bytes += (uint64_t)elems[i].num * message_size;
    Lease L;
    if (!acquire(L)) {
        t_last_error = cudaErrorNoDevice;
        memset(out, 0, out_bytes);
        return;
    }
    cudaStream_t s = use_non_default_stream ? L.q->stream : 0;
    cudaError_t e = run_sig_batch(L, s, sign, elems, num_elems, message_size, total_bytes, total_signatures,
                                  message_lens, key_offsets, sig_offsets, message_start_offsets, out);
    if (e != cudaSuccess) {
        fprintf(stderr, "libcuda-crypt: %s_many failed: %s\n", sign ? "sign" : "verify", cudaGetErrorString(e));
        cudaGetLastError();
        memset(out, 0, out_bytes);
    }
    t_last_error = (int)e;
}

}  // namespace

bool crypt_device_info(int dev, CryptDeviceInfo* out) {
    Device* D = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!init_locked() || dev < 0 || dev >= g_num_gpus) return false;
        D = &g_dev[dev];
    }
    const Tuning& T = tuning_for(*D);
    out->tables = D->tables;
    out->sms = D->sms;
    out->sig_threads = T.sig_threads;
    out->sig_blocks_per_sm = T.sig_blocks_per_sm;
    out->verify_window = T.verify_window;
    out->poh_warps = 4 * D->sms * T.poh_warps_per_smsp;
    return true;
}

extern "C" {

bool ed25519_init(void) {
    cudaFree(0);
    std::lock_guard<std::mutex> lk(g_mu);
    return init_locked();
}

void ed25519_set_verbose(bool val) { g_verbose.store(val); }

void poh_verify_many_set_verbose(bool val) { g_verbose.store(val); }

int gb300_crypt_last_error(void) { return t_last_error; }

void ed25519_verify_many(const gpu_Elems* elems, uint32_t num_elems, uint32_t message_size,
                         uint32_t total_packets, uint32_t total_signatures, const uint32_t* message_lens,
                         const uint32_t* public_key_offsets, const uint32_t* signature_offsets,
                         const uint32_t* message_start_offsets, uint8_t* out, uint8_t use_non_default_stream) {
    sig_many(false, elems, num_elems, message_size, total_packets, total_signatures, message_lens,
             public_key_offsets, signature_offsets, message_start_offsets, out, use_non_default_stream);
}

void ed25519_sign_many(const gpu_Elems* elems, uint32_t num_elems, uint32_t message_size,
                       uint32_t total_packets, uint32_t total_signatures, const uint32_t* message_lens,
                       const uint32_t* public_key_offsets, const uint32_t* private_key_offsets,
                       const uint32_t* message_start_offsets, uint8_t* signatures_out,
                       uint8_t use_non_default_stream) {
    sig_many(true, elems, num_elems, message_size, total_packets, total_signatures, message_lens,
             public_key_offsets, private_key_offsets, message_start_offsets, signatures_out,
             use_non_default_stream);
}

int poh_verify_many(uint8_t* hashes, const uint64_t* num_hashes_arr, size_t num_elems,
                    uint8_t use_non_default_stream) {
    LOG("Starting poh_verify_many: num_elems: %zu\n", num_elems);
    if (num_elems == 0) return 0;
    if (!hashes || !num_hashes_arr) return (int)cudaErrorInvalidValue;
    Lease L;
    if (!acquire(L)) return 1;
    Queue& Q = *L.q;
    cudaStream_t s = use_non_default_stream ? Q.stream : 0;
    const size_t hb = 32ull * num_elems, cb = 8ull * num_elems;
    auto run = [&]() -> cudaError_t {
        TRY(Q.d_data.ensure(hb + cb, s));
        TRY(Q.h_stage.ensure(hb + cb));
        uint8_t* st = static_cast<uint8_t*>(Q.h_stage.p);
        memcpy(st, hashes, hb);
        memcpy(st + hb, num_hashes_arr, cb);
        uint8_t* d = static_cast<uint8_t*>(Q.d_data.p);
        TRY(cudaMemcpyAsync(d, st, hb + cb, cudaMemcpyHostToDevice, s));
        TRY(launch_poh_verify(d, reinterpret_cast<const uint64_t*>(d + hb), num_elems, s));
        TRY(cudaMemcpyAsync(st, d, hb, cudaMemcpyDeviceToHost, s));
        TRY(cudaStreamSynchronize(s));
        memcpy(hashes, st, hb);
        return cudaSuccess;
    };
    cudaError_t e = run();
    if (e != cudaSuccess) {
        fprintf(stderr, "libcuda-crypt: poh_verify_many failed: %s\n", cudaGetErrorString(e));
        cudaGetLastError();
    }
    t_last_error = (int)e;
    return (int)e;
}

int cuda_host_register(void* ptr, size_t size, unsigned int flags) {
    return (int)cudaHostRegister(ptr, size, flags);
}

int cuda_host_unregister(void* ptr) { return (int)cudaHostUnregister(ptr); }

const char* ed25519_license(void) {
    return "GB300 libcuda-crypt: Ed25519 verify/sign and SHA-256 PoH verify for sm_103a. "
           "Drop-in for the libcuda-crypt.so interface of solana-perf-libs "
           "(Copyright (c) 2018 Solana Labs, Inc., Apache License 2.0).";
}

void ed25519_free_gpu_mem(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_num_gpus <= 0) return;
    int prev = -1;
    cudaGetDevice(&prev);
    for (int d = 0; d < g_num_gpus; d++) {
        cudaSetDevice(d);
        for (int k = 0; k < kQueues; k++) {
            std::lock_guard<std::mutex> ql(g_dev[d].q[k].mu);
            g_dev[d].q[k].release_buffers();
        }
    }
    if (prev >= 0) cudaSetDevice(prev);
}

int ed25519_create_seed(unsigned char* seed) {
    FILE* f = fopen("/dev/urandom", "rb");
    if (!f) return 1;
    size_t r = fread(seed, 1, 32, f);
    fclose(f);
    return r == 32 ? 0 : 1;
}

int ed25519_get_checked_scalar(unsigned char* out_scalar, const unsigned char* in_scalar) {
    if ((in_scalar[31] & 0xf0) != 0) return 1;
    memcpy(out_scalar, in_scalar, 32);
    return 0;
}

int gb300_ed25519_create_keypairs(const uint8_t* seeds, uint8_t* public_keys, uint8_t* private_keys,
                                  uint32_t num) {
    if (num == 0) return 0;
    Lease L;
    if (!acquire(L)) return t_last_error = (int)cudaErrorNoDevice;
    Queue& Q = *L.q;
    cudaStream_t s = Q.stream;
    auto run = [&]() -> cudaError_t {
        const size_t sb = 32ull * num, pb = 32ull * num, kb = 64ull * num;
        TRY(Q.d_data.ensure(sb + pb + kb, s));
        TRY(Q.h_stage.ensure(sb + pb + kb));
        uint8_t* st = static_cast<uint8_t*>(Q.h_stage.p);
        uint8_t* d = static_cast<uint8_t*>(Q.d_data.p);
        memcpy(st, seeds, sb);
        TRY(cudaMemcpyAsync(d, st, sb, cudaMemcpyHostToDevice, s));
        TRY(launch_ed25519_keypair(d, d + sb, d + sb + pb, num, L.dev->tables, s));
        TRY(cudaMemcpyAsync(st + sb, d + sb, pb + kb, cudaMemcpyDeviceToHost, s));
        TRY(cudaStreamSynchronize(s));
        memcpy(public_keys, st + sb, pb);
        memcpy(private_keys, st + sb + pb, kb);
        return cudaSuccess;
    };
    cudaError_t e = run();
    if (e != cudaSuccess) cudaGetLastError();
    return t_last_error = (int)e;
}

void ed25519_create_keypair(unsigned char* public_key, unsigned char* private_key, const unsigned char* seed) {
    gb300_ed25519_create_keypairs(seed, public_key, private_key, 1);
}

void ed25519_sign(unsigned char* signature, const unsigned char* message, size_t message_len,
                  const unsigned char* public_key, const unsigned char* private_key) {
    std::vector<uint8_t> img(96 + message_len);
    memcpy(img.data(), private_key, 64);
    memcpy(img.data() + 64, public_key, 32);
    if (message_len) memcpy(img.data() + 96, message, message_len);
    gpu_Elems e{img.data(), 1};
    uint32_t len = (uint32_t)message_len, pk = 64, sk = 0, mo = 96;
    sig_many(true, &e, 1, (uint32_t)img.size(), 1, 1, &len, &pk, &sk, &mo, signature, 1);
}

int ed25519_verify(const unsigned char* signature, const unsigned char* message, uint32_t message_len,
                   const unsigned char* public_key) {
    std::vector<uint8_t> img(96 + (size_t)message_len);
    memcpy(img.data(), signature, 64);
    memcpy(img.data() + 64, public_key, 32);
    if (message_len) memcpy(img.data() + 96, message, message_len);
    gpu_Elems e{img.data(), 1};
    uint32_t len = message_len, pk = 64, so = 0, mo = 96;
    uint8_t out = 0;
    sig_many(false, &e, 1, (uint32_t)img.size(), 1, 1, &len, &pk, &so, &mo, &out, 1);
    return out;
}

int ed25519_check_packed_ge_small_order(const unsigned char* packed_group_element) {
    Lease L;
    if (!acquire(L)) {
        t_last_error = (int)cudaErrorNoDevice;
        return 1;
    }
    Queue& Q = *L.q;
    cudaStream_t s = Q.stream;
    uint8_t result = 1;
    auto run = [&]() -> cudaError_t {
        TRY(Q.d_data.ensure(64, s));
        TRY(Q.h_stage.ensure(64));
        uint8_t* st = static_cast<uint8_t*>(Q.h_stage.p);
        uint8_t* d = static_cast<uint8_t*>(Q.d_data.p);
        memcpy(st, packed_group_element, 32);
        TRY(cudaMemcpyAsync(d, st, 32, cudaMemcpyHostToDevice, s));
        TRY(launch_check_small_order(d, d + 32, 1, L.dev->tables, s));
        TRY(cudaMemcpyAsync(st + 32, d + 32, 1, cudaMemcpyDeviceToHost, s));
        TRY(cudaStreamSynchronize(s));
        result = st[32];
        return cudaSuccess;
    };
    cudaError_t e = run();
    if (e != cudaSuccess) cudaGetLastError();
    t_last_error = (int)e;
    return e == cudaSuccess ? result : 1;
}

int gb300_ed25519_verify_device(const uint8_t* packets, uint64_t packets_len, const uint32_t* message_lens,
                                const uint32_t* public_key_offsets, const uint32_t* signature_offsets,
                                const uint32_t* message_start_offsets, uint32_t num, uint8_t* out,
                                void* stream) {
    if (num == 0) return 0;
    Device* D = current_device();
    if (!D) return (int)cudaErrorNoDevice;
    if (reinterpret_cast<uintptr_t>(packets) & 3u) return (int)cudaErrorMisalignedAddress;
    SigBatch b{packets, packets_len, message_lens, public_key_offsets, signature_offsets,
               message_start_offsets, num, out, D->tables};
    b.window = verify_window_if_tuned(*D);
    return (int)launch_ed25519_verify(b, static_cast<cudaStream_t>(stream));
}

int gb300_ed25519_verify_device_form(const uint8_t* packets, uint64_t packets_len, const uint32_t* message_lens,
                                     const uint32_t* public_key_offsets, const uint32_t* signature_offsets,
                                     const uint32_t* message_start_offsets, uint32_t num, uint8_t* out, int form,
                                     void* stream) {
    if (num == 0) return 0;
    if (form < 0 || form > 6) return (int)cudaErrorInvalidValue;
    Device* D = current_device();
    if (!D) return (int)cudaErrorNoDevice;
    if (reinterpret_cast<uintptr_t>(packets) & 3u) return (int)cudaErrorMisalignedAddress;
    SigBatch b{packets, packets_len, message_lens, public_key_offsets, signature_offsets,
               message_start_offsets, num, out, D->tables};
    b.window = form == 2 ? 4 : form == 3 ? 5 : form == 6 ? 0 : verify_window_if_tuned(*D);
    return (int)launch_ed25519_verify_form(b, static_cast<cudaStream_t>(stream),
                                           form == 1 ? kVerifyQuad : form == 4 ? kVerifyTrio : form == 5 ? kVerifyStaged : kVerifySingle);
}

int gb300_diag_half_scalars(const uint32_t* h, uint32_t num, uint32_t* out, void* stream) {
    if (num == 0) return 0;
    if (!current_device()) return (int)cudaErrorNoDevice;
    return (int)launch_half_scalars(h, num, out, static_cast<cudaStream_t>(stream));
}

int gb300_ed25519_sign_device(const uint8_t* packets, uint64_t packets_len, const uint32_t* message_lens,
                              const uint32_t* public_key_offsets, const uint32_t* private_key_offsets,
                              const uint32_t* message_start_offsets, uint32_t num, uint8_t* signatures_out,
                              void* stream) {
    if (num == 0) return 0;
    const CurveTables* T = tables_for_current_device();
    if (!T) return (int)cudaErrorNoDevice;
    if ((reinterpret_cast<uintptr_t>(packets) | reinterpret_cast<uintptr_t>(signatures_out)) & 3u)
        return (int)cudaErrorMisalignedAddress;
    SigBatch b{packets, packets_len, message_lens, public_key_offsets, private_key_offsets,
               message_start_offsets, num, signatures_out, T};
    return (int)launch_ed25519_sign(b, static_cast<cudaStream_t>(stream));
}

int gb300_ed25519_keypair_device(const uint8_t* seeds, uint8_t* public_keys, uint8_t* private_keys, uint32_t num,
                                 void* stream) {
    if (num == 0) return 0;
    const CurveTables* T = tables_for_current_device();
    if (!T) return (int)cudaErrorNoDevice;
    if ((reinterpret_cast<uintptr_t>(seeds) | reinterpret_cast<uintptr_t>(public_keys) |
         reinterpret_cast<uintptr_t>(private_keys)) & 3u)
        return (int)cudaErrorMisalignedAddress;
    return (int)launch_ed25519_keypair(seeds, public_keys, private_keys, num, T, static_cast<cudaStream_t>(stream));
}

int gb300_poh_verify_device(uint8_t* hashes, const uint64_t* num_hashes, uint64_t num_elems, void* stream) {
    if (num_elems == 0) return 0;
    if ((reinterpret_cast<uintptr_t>(hashes) & 15u) || (reinterpret_cast<uintptr_t>(num_hashes) & 7u))
        return (int)cudaErrorMisalignedAddress;
    return (int)launch_poh_verify(hashes, num_hashes, num_elems, static_cast<cudaStream_t>(stream));
}

int gb300_crypt_tuning(char* buf, size_t len) {
    Device* D = current_device();
    if (!D || !buf || len == 0) return 0;
    const Tuning& T = tuning_for(*D);
    int n = snprintf(buf, len,
                     "{\"device\": %d, \"sms\": %d, \"sig_threads\": %d, \"sig_blocks_per_sm\": %d, "
                     "\"verify_window\": %d, "
                     "\"sig_calibration_ms\": {\"half\": {\"64\": %.4f, \"128\": %.4f, \"256\": %.4f}, "
                     "\"w4\": {\"64\": %.4f, \"128\": %.4f, \"256\": %.4f}}, "
                     "\"sig_calibration_items\": %d, \"poh_warps_per_smsp\": %d, \"poh_paired\": %d, "
                     "\"poh_calibration_ms\": {\"single_1\": %.4f, \"single_2\": %.4f, \"paired_1\": %.4f, "
                     "\"paired_2\": %.4f}, \"poh_calibration_chains\": %d}",
                     D->id, D->sms, T.sig_threads, T.sig_blocks_per_sm, T.verify_window, T.sig_ms[0][0],
                     T.sig_ms[0][1], T.sig_ms[0][2], T.sig_ms[1][0], T.sig_ms[1][1], T.sig_ms[1][2],
                     T.calib_sigs, T.poh_warps_per_smsp, T.poh_form == kPohPair, T.poh_ms[0], T.poh_ms[1],
                     T.poh_ms[2], T.poh_ms[3], T.calib_chains);
    return n < 0 ? 0 : (n < (int)len ? n : (int)len - 1);
}

size_t gb300_poh_batch_workspace_size(uint64_t num_elems) { return poh_batch_workspace_size(num_elems); }

static int poh_batch_device_checks(const uint8_t* hashes, const uint64_t* num_hashes, uint64_t num_elems,
                                   const void* workspace, size_t workspace_bytes) {
    if (num_elems > 0xffffffffull) return (int)cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(hashes) & 15u) || (reinterpret_cast<uintptr_t>(num_hashes) & 7u) ||
        (reinterpret_cast<uintptr_t>(workspace) & 15u))
        return (int)cudaErrorMisalignedAddress;
    if (workspace_bytes < poh_batch_workspace_size(num_elems)) return (int)cudaErrorInvalidValue;
    return 0;
}

int gb300_poh_verify_batch_device(uint8_t* hashes, const uint64_t* num_hashes, uint64_t num_elems, void* workspace,
                                  size_t workspace_bytes, void* stream) {
    if (num_elems == 0) return 0;
    if (int rc = poh_batch_device_checks(hashes, num_hashes, num_elems, workspace, workspace_bytes)) return rc;
    Device* D = current_device();
    if (!D) return (int)cudaErrorNoDevice;
    const Tuning& T = tuning_for(*D);
    // the counts are in device memory: a paired tuning lets the device
    // choose between paired and single warps from them (kPohAuto), as
    // poh_host_batch_shape does from host counts
    return (int)launch_poh_batch(hashes, num_hashes, num_elems, workspace, 4 * D->sms * T.poh_warps_per_smsp,
                                 static_cast<cudaStream_t>(stream), T.poh_form == kPohPair ? kPohAuto : T.poh_form);
}

int gb300_poh_verify_batch_shape(uint8_t* hashes, const uint64_t* num_hashes, uint64_t num_elems, void* workspace,
                                 size_t workspace_bytes, int warps, int form, void* stream) {
    if (num_elems == 0) return 0;
    if (int rc = poh_batch_device_checks(hashes, num_hashes, num_elems, workspace, workspace_bytes)) return rc;
    if (form < kPohSingle || form > kPohAuto) return (int)cudaErrorInvalidValue;
    Device* D = current_device();
    if (!D) return (int)cudaErrorNoDevice;
    if (warps < 1 || warps > 64 * D->sms) return (int)cudaErrorInvalidValue;
    return (int)launch_poh_batch(hashes, num_hashes, num_elems, workspace, warps, static_cast<cudaStream_t>(stream),
                                 form);
}

// Launch shape of a ragged PoH batch whose counts the host holds.  The
// paired form runs a chain fastest (~1,900 cycles per hash on GB300) but
// keeps half its warps on the schedule; single warps, four per
// sub-partition, fill the ALU pipes (measured 16.2 Ghash/s against 10.7 for
// the paired batch at 77,824 chains).  Estimated makespans, in cycles:
//   paired  max(longest * 1900, total * 1900 / (64 SMs))    (2 pairs per SM)
//   single  max(longest * 2550, total * 77.5 / (4 SMs))     (4 warps per sub-partition)
// The single form is taken when its estimate is below 90 % of the paired
// one (a batch bounded by its total work, not by its longest chain);
// otherwise the tuned shape stays.
static void poh_host_batch_shape(const Tuning& T, int sms, const uint64_t* counts, size_t n, int* warps, int* form) {
    *warps = 4 * sms * T.poh_warps_per_smsp;
    *form = T.poh_form;
    if (T.poh_form != kPohPair) return;
    long double total = 0;
    uint64_t longest = 0;
    for (size_t i = 0; i < n; i++) {
        total += (long double)counts[i];
        longest = counts[i] > longest ? counts[i] : longest;
    }
    const long double pair = std::max((long double)longest * 1900.0L, total * 1900.0L / (64.0L * sms));
    const long double single = std::max((long double)longest * 2550.0L, total * 77.5L / (4.0L * sms));
    if (single < 0.9L * pair) {
        *warps = 16 * sms;
        *form = kPohSingle;
    }
}

int gb300_poh_verify_batch(uint8_t* hashes, const uint64_t* num_hashes_arr, size_t num_elems) {
    if (num_elems == 0) return 0;
    if (!hashes || !num_hashes_arr || num_elems > 0xffffffffull) return (int)cudaErrorInvalidValue;
    Lease L;
    if (!acquire(L)) return 1;
    const Tuning& T = tuning_for(*L.dev);
    Queue& Q = *L.q;
    cudaStream_t s = Q.stream;
    const size_t hb = 32ull * num_elems, cb = 8ull * num_elems, wb = poh_batch_workspace_size(num_elems);
    int warps = 0, form = 0;
    poh_host_batch_shape(T, L.dev->sms, num_hashes_arr, num_elems, &warps, &form);
    auto run = [&]() -> cudaError_t {
        TRY(Q.d_data.ensure(hb + cb, s));
        TRY(Q.d_scratch.ensure(wb, s));
        TRY(Q.h_stage.ensure(hb + cb));
        uint8_t* st = static_cast<uint8_t*>(Q.h_stage.p);
        memcpy(st, hashes, hb);
        memcpy(st + hb, num_hashes_arr, cb);
        uint8_t* d = static_cast<uint8_t*>(Q.d_data.p);
        const uint64_t* dc = reinterpret_cast<const uint64_t*>(d + hb);
        TRY(cudaMemcpyAsync(d, st, hb + cb, cudaMemcpyHostToDevice, s));
        std::vector<uint64_t> key = {num_elems, (uint64_t)(uintptr_t)d, (uint64_t)(uintptr_t)Q.d_scratch.p,
                                     (uint64_t)warps, (uint64_t)form};
        TRY(run_graph(Q.g_poh, key, s, [&](cudaStream_t cs) {
            return launch_poh_batch(d, dc, num_elems, Q.d_scratch.p, warps, cs, form);
        }));
        TRY(cudaMemcpyAsync(st, d, hb, cudaMemcpyDeviceToHost, s));
        TRY(cudaStreamSynchronize(s));
        memcpy(hashes, st, hb);
        return cudaSuccess;
    };
    cudaError_t e = run();
    if (e != cudaSuccess) {
        fprintf(stderr, "libcuda-crypt: gb300_poh_verify_batch failed: %s\n", cudaGetErrorString(e));
        cudaGetLastError();
    }
    return t_last_error = (int)e;
}

// ---- Solana ledger entries (poh_entries.cu) ----

size_t gb300_poh_entries_workspace_size(uint64_t num_entries) { return poh_entries_workspace_size(num_entries); }

int gb300_poh_verify_entries_device(const uint8_t* start_hashes, const uint64_t* num_hashes, const uint8_t* mixins,
                                    const uint8_t* has_mixin, const uint8_t* expected, uint64_t num_entries,
                                    uint8_t* ok, uint8_t* out_hashes, void* workspace, size_t workspace_bytes,
                                    void* stream) {
    if (num_entries == 0) return 0;
    if (!start_hashes || !num_hashes || !mixins || !has_mixin || !expected || !ok || !workspace ||
        num_entries > 0xffffffffull)
        return (int)cudaErrorInvalidValue;
    if (workspace_bytes < poh_entries_workspace_size(num_entries)) return (int)cudaErrorInvalidValue;
    if (((reinterpret_cast<uintptr_t>(start_hashes) | reinterpret_cast<uintptr_t>(mixins) |
          reinterpret_cast<uintptr_t>(expected) | reinterpret_cast<uintptr_t>(out_hashes) |
          reinterpret_cast<uintptr_t>(workspace)) & 15u) ||
        (reinterpret_cast<uintptr_t>(num_hashes) & 7u))
        return (int)cudaErrorMisalignedAddress;
    Device* D = current_device();
    if (!D) return (int)cudaErrorNoDevice;
    const Tuning& T = tuning_for(*D);
    return (int)launch_poh_verify_entries(start_hashes, num_hashes, mixins, has_mixin, expected, num_entries, ok,
                                          out_hashes, workspace, 4 * D->sms * T.poh_warps_per_smsp,
                                          static_cast<cudaStream_t>(stream));
}

int gb300_poh_verify_entries(const uint8_t* start_hashes, const uint64_t* num_hashes, const uint8_t* mixins,
                             const uint8_t* has_mixin, const uint8_t* expected, size_t num_entries, uint8_t* ok) {
    if (num_entries == 0) return 0;
    if (!start_hashes || !num_hashes || !mixins || !has_mixin || !expected || !ok || num_entries > 0xffffffffull)
        return t_last_error = (int)cudaErrorInvalidValue;
    Lease L;
    if (!acquire(L)) return 1;
    const Tuning& T = tuning_for(*L.dev);
    Queue& Q = *L.q;
    cudaStream_t s = Q.stream;
    const uint64_t n = num_entries;
    // staging / device layout: start | expected | mixins | counts | flags
    const size_t hb = 32 * n, cb = 8 * n, in_bytes = 3 * hb + cb + n;
    auto run = [&]() -> cudaError_t {
        TRY(Q.d_data.ensure(round_up(in_bytes, 256), s));
        TRY(Q.d_scratch.ensure(poh_entries_workspace_size(n), s));
        TRY(Q.d_out.ensure(n, s));
        TRY(Q.h_stage.ensure(in_bytes));
        uint8_t* st = static_cast<uint8_t*>(Q.h_stage.p);
        memcpy(st, start_hashes, hb);
        memcpy(st + hb, expected, hb);
        memcpy(st + 2 * hb, mixins, hb);
        memcpy(st + 3 * hb, num_hashes, cb);
        memcpy(st + 3 * hb + cb, has_mixin, n);
        uint8_t* d = static_cast<uint8_t*>(Q.d_data.p);
        TRY(cudaMemcpyAsync(d, st, in_bytes, cudaMemcpyHostToDevice, s));
        TRY(launch_poh_verify_entries(d, reinterpret_cast<const uint64_t*>(d + 3 * hb), d + 2 * hb, d + 3 * hb + cb,
                                      d + hb, n, static_cast<uint8_t*>(Q.d_out.p), nullptr, Q.d_scratch.p,
                                      4 * L.dev->sms * T.poh_warps_per_smsp, s));
        TRY(cudaMemcpyAsync(st, Q.d_out.p, n, cudaMemcpyDeviceToHost, s));
        TRY(cudaStreamSynchronize(s));
        memcpy(ok, st, n);
        return cudaSuccess;
    };
    cudaError_t e = run();
    if (e != cudaSuccess) {
        fprintf(stderr, "libcuda-crypt: gb300_poh_verify_entries failed: %s\n", cudaGetErrorString(e));
        cudaGetLastError();
    }
    return t_last_error = (int)e;
}

int gb300_poh_record_device(uint8_t* hashes, uint64_t num_chains, const uint64_t* first, uint64_t num_entries,
                            const uint64_t* num_hashes, const uint8_t* mixins, const uint8_t* has_mixin,
                            uint8_t* entry_hashes, void* stream) {
    if (num_chains == 0) return 0;
    if (!hashes || !first || !num_hashes || !mixins || !has_mixin || !entry_hashes) return (int)cudaErrorInvalidValue;
    if (((reinterpret_cast<uintptr_t>(hashes) | reinterpret_cast<uintptr_t>(mixins) |
          reinterpret_cast<uintptr_t>(entry_hashes)) & 15u) ||
        ((reinterpret_cast<uintptr_t>(first) | reinterpret_cast<uintptr_t>(num_hashes)) & 7u))
        return (int)cudaErrorMisalignedAddress;
    if (!current_device()) return (int)cudaErrorNoDevice;
    return (int)launch_poh_record(hashes, num_chains, first, num_entries, num_hashes, mixins, has_mixin, entry_hashes,
                                  static_cast<cudaStream_t>(stream));
}

int gb300_poh_record(uint8_t* hashes, size_t num_chains, const uint64_t* first, const uint64_t* num_hashes,
                     const uint8_t* mixins, const uint8_t* has_mixin, uint8_t* entry_hashes) {
    if (num_chains == 0) return 0;
    if (!hashes || !first || !num_hashes || !mixins || !has_mixin || !entry_hashes)
        return t_last_error = (int)cudaErrorInvalidValue;
    // the chains' entry ranges must be well formed before anything is copied
    if (first[0] != 0) return t_last_error = (int)cudaErrorInvalidValue;
    for (size_t c = 0; c < num_chains; c++)
        if (first[c + 1] < first[c]) return t_last_error = (int)cudaErrorInvalidValue;
    const uint64_t ne = first[num_chains];
    if (ne > 0xffffffffull) return t_last_error = (int)cudaErrorInvalidValue;
    Lease L;
    if (!acquire(L)) return 1;
    Queue& Q = *L.q;
    cudaStream_t s = Q.stream;
    const uint64_t C = num_chains, E = ne ? ne : 1;
    // staging / device layout: chain hashes | mixins | entry hashes (out) | first | counts | flags
    const size_t hc = 32 * C, he = 32 * E, fb = 8 * (C + 1), cb = 8 * E;
    const size_t total = hc + 2 * he + fb + cb + E;
    auto run = [&]() -> cudaError_t {
        TRY(Q.d_data.ensure(round_up(total, 256), s));
        TRY(Q.h_stage.ensure(total));
        uint8_t* st = static_cast<uint8_t*>(Q.h_stage.p);
        memcpy(st, hashes, hc);
        if (ne) {
            memcpy(st + hc, mixins, 32 * ne);
            memcpy(st + hc + 2 * he + fb, num_hashes, 8 * ne);
            memcpy(st + hc + 2 * he + fb + cb, has_mixin, ne);
        }
        memcpy(st + hc + 2 * he, first, fb);
        uint8_t* d = static_cast<uint8_t*>(Q.d_data.p);
        TRY(cudaMemcpyAsync(d, st, total, cudaMemcpyHostToDevice, s));
        TRY(launch_poh_record(d, C, reinterpret_cast<const uint64_t*>(d + hc + 2 * he), ne,
                              reinterpret_cast<const uint64_t*>(d + hc + 2 * he + fb), d + hc,
                              d + hc + 2 * he + fb + cb, d + hc + he, s));
        TRY(cudaMemcpyAsync(st, d, hc + 2 * he, cudaMemcpyDeviceToHost, s));
        TRY(cudaStreamSynchronize(s));
        memcpy(hashes, st, hc);
        if (ne) memcpy(entry_hashes, st + hc + he, 32 * ne);
        return cudaSuccess;
    };
    cudaError_t e = run();
    if (e != cudaSuccess) {
        fprintf(stderr, "libcuda-crypt: gb300_poh_record failed: %s\n", cudaGetErrorString(e));
        cudaGetLastError();
    }
    return t_last_error = (int)e;
}

int gb300_ed25519_batch_device(const uint8_t* packets, uint64_t packets_len, const uint32_t* v_message_lens,
                               const uint32_t* v_public_key_offsets, const uint32_t* v_signature_offsets,
                               const uint32_t* v_message_start_offsets, uint32_t nv, uint8_t* v_out,
                               const uint32_t* s_message_lens, const uint32_t* s_public_key_offsets,
                               const uint32_t* s_private_key_offsets, const uint32_t* s_message_start_offsets,
                               uint32_t ns, uint8_t* s_out, uint32_t* queue_word, void* stream) {
    if (nv == 0 && ns == 0) return 0;
    if ((reinterpret_cast<uintptr_t>(packets) | reinterpret_cast<uintptr_t>(queue_word)) & 3u)
        return (int)cudaErrorMisalignedAddress;
    if (ns && (reinterpret_cast<uintptr_t>(s_out) & 3u)) return (int)cudaErrorMisalignedAddress;
    Device* D = current_device();
    if (!D) return (int)cudaErrorNoDevice;
    const Tuning& T = tuning_for(*D);
    SigWork w;
    w.v = SigBatch{packets, packets_len, v_message_lens, v_public_key_offsets, v_signature_offsets,
                   v_message_start_offsets, nv, v_out, D->tables};
    w.s = SigBatch{packets, packets_len, s_message_lens, s_public_key_offsets, s_private_key_offsets,
                   s_message_start_offsets, ns, s_out, D->tables};
    w.sign_base = (nv + 31u) / 32u * 32u;
    w.total_chunks = (w.sign_base + ns + 31u) / 32u;
    w.next = queue_word;
    w.v.window = T.verify_window;
    return (int)launch_sig_batch(w, T.sig_threads, T.sig_blocks_per_sm, D->sms, static_cast<cudaStream_t>(stream));
}

int gb300_ed25519_batch(const gb300_sig_job* jobs, uint32_t num_jobs) {
    if (num_jobs == 0) return 0;
    if (!jobs) return t_last_error = (int)cudaErrorInvalidValue;
    uint64_t nv = 0, ns = 0, total = 0;
    bool all_locked = true;
    for (uint32_t j = 0; j < num_jobs; j++) {
        const gb300_sig_job& J = jobs[j];
        if (J.num == 0) continue;
        if (!J.message_lens || !J.public_key_offsets || !J.key_offsets || !J.message_start_offsets || !J.out ||
            (J.packets_len && !J.packets) || J.kind > 1)
            return t_last_error = (int)cudaErrorInvalidValue;
        (J.kind == 0 ? nv : ns) += J.num;
        total += J.packets_len;
        if (J.packets_len && all_locked) all_locked = is_page_locked(J.packets);
    }
    if (nv + ns == 0) return 0;
    if (total >= 0xfffffff0ull || nv + ns > 0x7fffffffull) return t_last_error = (int)cudaErrorInvalidValue;
    Lease L;
    if (!acquire(L)) return t_last_error = (int)cudaErrorNoDevice;
    const Tuning& T = tuning_for(*L.dev);
    Queue& Q = *L.q;
    cudaStream_t s = Q.stream;
    auto run = [&]() -> cudaError_t {
        // verdicts, then signatures from a 64-byte boundary (32-bit stores)
        const size_t sig_out_off = round_up(nv, 64);
        const size_t idx_bytes = 16ull * (nv + ns), out_bytes = sig_out_off + 64ull * ns;
        const size_t pk_off = round_up(idx_bytes, 256);
        TRY(Q.d_data.ensure(total + 16, s));
        TRY(Q.d_index.ensure(idx_bytes, s));
        TRY(Q.d_out.ensure(out_bytes, s));
        TRY(Q.d_scratch.ensure(256, s));
        TRY(Q.h_stage.ensure(pk_off + (all_locked ? 0 : total)));
        TRY(Q.h_out.ensure(out_bytes));
        uint32_t* hv = static_cast<uint32_t*>(Q.h_stage.p);
        uint32_t* hs = hv + 4 * nv;
        uint8_t* img = static_cast<uint8_t*>(Q.h_stage.p) + pk_off;
        uint8_t* dpk = static_cast<uint8_t*>(Q.d_data.p);
        uint64_t base = 0, iv = 0, is = 0;
        std::vector<gb300::CopyPiece> pcs;
        for (uint32_t j = 0; j < num_jobs; j++) {
            const gb300_sig_job& J = jobs[j];
            if (J.num == 0) continue;
            uint32_t* h = J.kind == 0 ? hv : hs;
            const uint64_t cnt = J.kind == 0 ? nv : ns;
            uint64_t& pos = J.kind == 0 ? iv : is;
            const uint64_t key_len = 64;
            for (uint32_t i = 0; i < J.num; i++) {
                const uint64_t m = J.message_lens[i], po = J.public_key_offsets[i], ko = J.key_offsets[i],
                               mo = J.message_start_offsets[i];
                const bool ok = po + 32 <= J.packets_len && ko + key_len <= J.packets_len && mo + m <= J.packets_len;
                h[pos + i] = ok ? (uint32_t)m : 0xffffffffu;         // an out-of-range item fails on the GPU
                h[cnt + pos + i] = ok ? (uint32_t)(base + po) : 0u;
                h[2 * cnt + pos + i] = ok ? (uint32_t)(base + ko) : 0u;
                h[3 * cnt + pos + i] = ok ? (uint32_t)(base + mo) : 0u;
            }
            if (J.packets_len) {
                if (all_locked)
                    TRY(cudaMemcpyAsync(dpk + base, J.packets, J.packets_len, cudaMemcpyHostToDevice, s));
                else
                    pcs.push_back({img + base, J.packets, J.packets_len});
            }
            pos += J.num;
            base += J.packets_len;
        }
        gb300::CopyPool::copy(pcs.data(), pcs.size());
        TRY(cudaMemcpyAsync(Q.d_index.p, Q.h_stage.p, idx_bytes, cudaMemcpyHostToDevice, s));
        if (!all_locked && total) TRY(cudaMemcpyAsync(dpk, img, total, cudaMemcpyHostToDevice, s));
        const uint32_t* dv = static_cast<const uint32_t*>(Q.d_index.p);
        const uint32_t* ds = dv + 4 * nv;
        uint8_t* dout = static_cast<uint8_t*>(Q.d_out.p);
        SigWork w;
        w.v = SigBatch{dpk, total, dv, dv + nv, dv + 2 * nv, dv + 3 * nv, (uint32_t)nv, dout, L.dev->tables};
        w.s = SigBatch{dpk, total, ds, ds + ns, ds + 2 * ns, ds + 3 * ns, (uint32_t)ns, dout + sig_out_off,
                       L.dev->tables};
        w.sign_base = (uint32_t)((nv + 31) / 32 * 32);
        w.total_chunks = (uint32_t)((w.sign_base + ns + 31) / 32);
        w.next = static_cast<uint32_t*>(Q.d_scratch.p);
        w.v.window = T.verify_window;
        std::vector<uint64_t> key = {nv, ns, total, (uint64_t)(uintptr_t)dpk, (uint64_t)(uintptr_t)dv,
                                     (uint64_t)(uintptr_t)dout, (uint64_t)(uintptr_t)w.next,
                                     (uint64_t)T.sig_threads, (uint64_t)T.sig_blocks_per_sm,
                                     (uint64_t)T.verify_window};
        const int sms = L.dev->sms;
        TRY(run_graph(Q.g_sig, key, s, [&](cudaStream_t cs) {
            return launch_sig_batch(w, T.sig_threads, T.sig_blocks_per_sm, sms, cs);
        }));
        TRY(cudaMemcpyAsync(Q.h_out.p, dout, out_bytes, cudaMemcpyDeviceToHost, s));
        TRY(cudaStreamSynchronize(s));
        const uint8_t* ho = static_cast<const uint8_t*>(Q.h_out.p);
        uint64_t ov = 0, os = 0;
        for (uint32_t j = 0; j < num_jobs; j++) {
            const gb300_sig_job& J = jobs[j];
            if (J.num == 0) continue;
            if (J.kind == 0) {
                memcpy(J.out, ho + ov, J.num);
                ov += J.num;
            } else {
                memcpy(J.out, ho + sig_out_off + 64 * os, 64ull * J.num);
                os += J.num;
            }
        }
        return cudaSuccess;
    };
    cudaError_t e = run();
    if (e != cudaSuccess) {
        fprintf(stderr, "libcuda-crypt: gb300_ed25519_batch failed: %s\n", cudaGetErrorString(e));
        cudaGetLastError();
        for (uint32_t j = 0; j < num_jobs; j++)
            if (jobs[j].out && jobs[j].num) memset(jobs[j].out, 0, jobs[j].kind == 0 ? jobs[j].num : 64ull * jobs[j].num);
    }
    return t_last_error = (int)e;
}

// ---------------------------------------------------------------------------
// Solana wire-format packet batches (gb300_packets.h; kernels in packets.cu).

size_t gb300_packets_workspace_size(uint32_t num_packets, uint64_t stride) {
    return packets_workspace_size(num_packets, stride);
}

uint64_t gb300_packets_signature_capacity(uint32_t num_packets, uint64_t stride) {
    return packets_signature_capacity(num_packets, stride);
}

int gb300_packets_extract_offsets_device(const uint8_t* packets, uint64_t stride, uint32_t num_packets,
                                         const uint32_t* packet_lens, void* workspace, size_t workspace_bytes,
                                         uint32_t* message_lens, uint32_t* public_key_offsets,
                                         uint32_t* signature_offsets, uint32_t* message_start_offsets,
                                         uint32_t* sig_counts, uint32_t* total_signatures, void* stream) {
    return (int)launch_packets_extract(packets, stride, num_packets, packet_lens, workspace, workspace_bytes,
                                       message_lens, public_key_offsets, signature_offsets, message_start_offsets,
                                       sig_counts, total_signatures, static_cast<cudaStream_t>(stream));
}

int gb300_ed25519_verify_packets_device(const uint8_t* packets, uint64_t stride, uint32_t num_packets,
                                        const uint32_t* packet_lens, void* workspace, size_t workspace_bytes,
                                        uint8_t* packet_out, uint32_t* sig_counts, void* stream) {
    if (num_packets == 0) return 0;
    Device* D = current_device();
    if (!D) return (int)cudaErrorNoDevice;
    const Tuning& T = tuning_for(*D);
    return (int)launch_packets_verify(packets, stride, num_packets, packet_lens, workspace, workspace_bytes,
                                      packet_out, sig_counts, D->tables, T.sig_threads, T.sig_blocks_per_sm,
                                      D->sms, static_cast<cudaStream_t>(stream), T.verify_window);
}

int gb300_ed25519_verify_packets(const gpu_Elems* elems, uint32_t num_elems, uint32_t stride,
                                 const uint32_t* packet_lens, uint8_t* packet_out, uint32_t* sig_counts) {
    uint64_t np = 0;
    if (num_elems && !elems) return t_last_error = (int)cudaErrorInvalidValue;
    for (uint32_t i = 0; i < num_elems; i++) np += elems[i].num;
    if (np == 0) return 0;
    if (!packet_lens || !packet_out || stride == 0) return t_last_error = (int)cudaErrorInvalidValue;
    const uint64_t total = np * stride;
    if (np > 0xffffffffull || total > 0xffffffffull) {
        memset(packet_out, 0, np);
        if (sig_counts) memset(sig_counts, 0, 4 * np);
        return t_last_error = (int)cudaErrorInvalidValue;
    }
    const uint32_t n = (uint32_t)np;
    Lease L;
    if (!acquire(L)) {
        memset(packet_out, 0, np);
        if (sig_counts) memset(sig_counts, 0, 4 * np);
        return t_last_error = (int)cudaErrorNoDevice;
    }
    const Tuning& T = tuning_for(*L.dev);
    Queue& Q = *L.q;
    cudaStream_t s = Q.stream;
    auto run = [&]() -> cudaError_t {
        bool all_locked = true;
        for (uint32_t i = 0; i < num_elems && all_locked; i++)
            if (elems[i].num) all_locked = is_page_locked(elems[i].elems);
        const size_t lens_bytes = 4ull * n;
        const size_t pk_off = round_up(lens_bytes, 256);
        const size_t out_off = round_up(n, 256);               // d_out: verdicts, then counts
        const size_t out_bytes = out_off + 4ull * n;
        const size_t ws_bytes = packets_workspace_size(n, stride);
        TRY(Q.d_data.ensure(round_up(total, 256) + lens_bytes, s));
        TRY(Q.d_scratch.ensure(ws_bytes, s));
        TRY(Q.d_out.ensure(out_bytes, s));
        TRY(Q.h_stage.ensure(pk_off + (all_locked ? 0 : total)));
        TRY(Q.h_out.ensure(out_bytes));
        uint8_t* dpk = static_cast<uint8_t*>(Q.d_data.p);
        uint32_t* dlens = reinterpret_cast<uint32_t*>(dpk + round_up(total, 256));
        memcpy(Q.h_stage.p, packet_lens, lens_bytes);
        TRY(cudaMemcpyAsync(dlens, Q.h_stage.p, lens_bytes, cudaMemcpyHostToDevice, s));
        uint64_t cur = 0;
        uint8_t* img = static_cast<uint8_t*>(Q.h_stage.p) + pk_off;
        std::vector<gb300::CopyPiece> pcs;
        for (uint32_t i = 0; i < num_elems; i++) {
            const uint64_t b = (uint64_t)elems[i].num * stride;
            if (!b) continue;
            if (all_locked) TRY(cudaMemcpyAsync(dpk + cur, elems[i].elems, b, cudaMemcpyHostToDevice, s));
            else pcs.push_back({img + cur, elems[i].elems, b});
            cur += b;
        }
        gb300::CopyPool::copy(pcs.data(), pcs.size());
        if (!all_locked) TRY(cudaMemcpyAsync(dpk, img, total, cudaMemcpyHostToDevice, s));
        uint8_t* dout = static_cast<uint8_t*>(Q.d_out.p);
        uint32_t* dcnt = reinterpret_cast<uint32_t*>(dout + out_off);
        std::vector<uint64_t> key = {1, n, stride, (uint64_t)(uintptr_t)dpk, (uint64_t)(uintptr_t)Q.d_scratch.p,
                                     (uint64_t)(uintptr_t)dout, (uint64_t)T.sig_threads, (uint64_t)T.verify_window};
        TRY(run_graph(Q.g_pkt, key, s, [&](cudaStream_t cs) {
            return launch_packets_verify(dpk, stride, n, dlens, Q.d_scratch.p, ws_bytes, dout, dcnt, L.dev->tables,
                                         T.sig_threads, T.sig_blocks_per_sm, L.dev->sms, cs, T.verify_window);
        }));
        TRY(cudaMemcpyAsync(Q.h_out.p, dout, out_bytes, cudaMemcpyDeviceToHost, s));
        TRY(cudaStreamSynchronize(s));
        memcpy(packet_out, Q.h_out.p, n);
        if (sig_counts) memcpy(sig_counts, static_cast<uint8_t*>(Q.h_out.p) + out_off, 4ull * n);
        return cudaSuccess;
    };
    cudaError_t e = run();
    if (e != cudaSuccess) {
        fprintf(stderr, "libcuda-crypt: gb300_ed25519_verify_packets failed: %s\n", cudaGetErrorString(e));
        cudaGetLastError();
        memset(packet_out, 0, np);
        if (sig_counts) memset(sig_counts, 0, 4 * np);
    }
    return t_last_error = (int)e;
}

}  // extern "C"
