// C ABI of libcuda-crypt.so: the reference's entry points (include/ed25519.h,
// include/poh_verify.h) over a pool of GPU queues.
//
// Replaces the reference's host drivers and context pool
// (src/cuda-ecc-ed25519/gpu_ctx.cu:8-165, verify.cu:240-340,
// sign.cu:76-145, src/cuda-poh-verify/poh_verify.cu:29-144).
// Same pool shape (up to 8 GPUs x 8 queues, round-robin, one lock per
// queue, grow-only device buffers) shared by every entry point, plus:
//   * a grow-only page-locked staging buffer per queue: the four per-
//     signature index arrays and the packets go to the GPU in one copy
//     (packets that the caller page-locked with cuda_host_register are
//     copied straight from the caller's memory instead);
//   * argument checks and error codes instead of assert() aborts;
//   * device tables (curve constants, basepoint multiples) built on the GPU
//     when the pool is created.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "ed25519.h"
#include "poh_verify.h"
#include "kernels.h"
#include "tables.cuh"

namespace {

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

size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (p && bytes <= cap) return cudaSuccess;
        release();
        size_t want = round_up(bytes < 4096 ? 4096 : bytes + bytes / 4, 4096);
        cudaError_t e = cudaMalloc(&p, want);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        cap = want;
        return cudaSuccess;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct HostBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (p && bytes <= cap) return cudaSuccess;
        release();
        size_t want = round_up(bytes < 4096 ? 4096 : bytes + bytes / 4, 4096);
        cudaError_t e = cudaMallocHost(&p, want);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        cap = want;
        return cudaSuccess;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

struct Queue {
    std::mutex mu;
    cudaStream_t stream = nullptr;
    DevBuf d_data, d_index, d_out;
    HostBuf h_stage, h_out;
    void release_buffers() {
        d_data.release();
        d_index.release();
        d_out.release();
        h_stage.release();
        h_out.release();
    }
};

struct Device {
    int id = -1;
    CurveTables* tables = nullptr;
    Queue q[kQueues];
    uint32_t next_queue = 0;
};

std::mutex g_mu;
int g_num_gpus = -1;  // -1: not initialised yet
Device g_dev[kMaxGpus];
uint32_t g_next_gpu = 0;

bool init_locked() {
    if (g_num_gpus >= 0) return g_num_gpus > 0;
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
        bool ok = true;
        for (int k = 0; k < kQueues && ok; k++)
            ok = cudaStreamCreateWithFlags(&D.q[k].stream, cudaStreamNonBlocking) == cudaSuccess;
        if (ok) ok = crypt_tables_create(&D.tables, D.q[0].stream) == cudaSuccess;
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

// Round-robin (gpu, queue) pick, then the queue's lock (reference
// gpu_ctx.cu:46-73).
bool acquire(Lease& L) {
    std::unique_lock<std::mutex> lk(g_mu);
    if (!init_locked()) return false;
    Device& D = g_dev[g_next_gpu % (uint32_t)g_num_gpus];
    g_next_gpu++;
    Queue& Q = D.q[D.next_queue % kQueues];
    D.next_queue++;
    lk.unlock();
    Q.mu.lock();
    L.dev = &D;
    L.q = &Q;
    cudaSetDevice(D.id);
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

    TRY(Q.d_data.ensure(total_bytes + 16));
    TRY(Q.d_index.ensure(idx_bytes));
    TRY(Q.d_out.ensure(out_bytes));
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
        uint64_t cur = 0;
        for (uint32_t i = 0; i < num_elems; i++) {
            uint64_t b = (uint64_t)elems[i].num * message_size;
            if (b) memcpy(img + cur, elems[i].elems, b);
            cur += b;
        }
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
        TRY(Q.d_data.ensure(hb + cb));
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
        TRY(Q.d_data.ensure(sb + pb + kb));
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
        TRY(Q.d_data.ensure(64));
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
    const CurveTables* T = tables_for_current_device();
    if (!T) return (int)cudaErrorNoDevice;
    if (reinterpret_cast<uintptr_t>(packets) & 3u) return (int)cudaErrorMisalignedAddress;
    SigBatch b{packets, packets_len, message_lens, public_key_offsets, signature_offsets,
               message_start_offsets, num, out, T};
    return (int)launch_ed25519_verify(b, static_cast<cudaStream_t>(stream));
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

}  // extern "C"
