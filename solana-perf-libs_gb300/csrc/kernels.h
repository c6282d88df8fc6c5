// Launch descriptors and host-side launch functions for the device kernels.
// Shared by the C-ABI layer (crypt_api.cu) and the kernel translation units.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

struct CurveTables;

// One batch of signatures over one contiguous device packet buffer, with the
// reference's per-signature arrays (src/cuda-ecc-ed25519/verify.cu:240-258):
// message length, and absolute byte offsets of the public key, signature and
// message start inside the buffer.
struct SigBatch {
    const uint8_t* packets;       // device
    uint64_t packets_len;         // bytes; reads past it are refused per item
    const uint32_t* message_lens;
    const uint32_t* public_key_offsets;
    const uint32_t* signature_offsets;      // for signing: private key offsets
    const uint32_t* message_start_offsets;
    uint32_t n;
    uint8_t* out;                 // verify: n verdict bytes; sign: n*64 bytes
    const CurveTables* tables;
    int window = 0;               // verify, one lane per signature: signed window width of h (4 or 5), or 0
                                  // for half-size scalars (the autotuner's choice)
};

// Kernels are loaded on the current device when these run, rather than at
// their first launch.  Under lazy module loading (CUDA's default) a kernel's
// first launch loads it, and that load can wait for unrelated kernels that
// are running: in the served loop a first-used signature kernel waited up to
// hundreds of ms for a PoH launch.  cudaFuncGetAttributes loads a function.
template <class... K>
inline cudaError_t load_kernels(K... k) {
    cudaError_t e = cudaSuccess;
    cudaFuncAttributes a;
    ((e = (e == cudaSuccess ? cudaFuncGetAttributes(&a, k) : e)), ...);
    return e;
}
cudaError_t preload_verify_kernels();
cudaError_t preload_sign_kernels();
cudaError_t preload_poh_kernels();
cudaError_t preload_poh_batch_kernels();
cudaError_t preload_sig_batch_kernels();
cudaError_t preload_packets_kernels();

// Ed25519 verify: out[i] = 1 if signature i is valid under the reference's
// acceptance rules, else 0.  Forms: one thread per signature, or four lanes
// per signature (lower latency on batches that do not fill the GPU).
enum VerifyForm : int { kVerifySingle = 0, kVerifyQuad = 1, kVerifyTrio = 2, kVerifyStaged = 3 };
cudaError_t launch_ed25519_verify(const SigBatch& b, cudaStream_t s);
cudaError_t launch_ed25519_verify_form(const SigBatch& b, cudaStream_t s, int form);

// Ed25519 sign: out[64*i ..] = R || S.  The 64-byte private key (clamped a,
// then the nonce prefix) sits at signature_offsets[i].
cudaError_t launch_ed25519_sign(const SigBatch& b, cudaStream_t s);

// Keypairs from 32-byte seeds (reference keypair.cu:6-16).
cudaError_t launch_ed25519_keypair(const uint8_t* seeds, uint8_t* pk, uint8_t* sk, uint32_t n,
                                   const CurveTables* tables, cudaStream_t s);

// 0 = decodes and has order not dividing 4 (reference verify.cu:88-103).
// The half-size scalars of n values h < L (verify_trio.cuh, half_scalar.cuh):
// 18 words per value into out (diagnostic; gb300_diag.h).
cudaError_t launch_half_scalars(const uint32_t* h, uint32_t n, uint32_t* out, cudaStream_t s);
cudaError_t launch_check_small_order(const uint8_t* points, uint8_t* out, uint32_t n,
                                     const CurveTables* tables, cudaStream_t s);

// PoH: hashes[32*i..] <- SHA-256^num_hashes[i] (hashes[32*i..]), in place.
cudaError_t launch_poh_verify(uint8_t* hashes, const uint64_t* num_hashes, uint64_t n, cudaStream_t s);

// Ragged PoH batch in one persistent launch (poh_batch.cu): entries ordered
// longest first, `warps` resident warps refilling lanes from a queue.
// `workspace` holds poh_batch_workspace_size(n) bytes of device memory.
enum PohBatchForm : int {
    kPohSingle = 0,         // one warp per 32 chains, one warp per block
    kPohPackedSingle = 1,   // one warp per 32 chains, four warps per block (fewer SMs)
    kPohPair = 2,           // schedule warp + round warp per 32 chains, one pair per block
    kPohPackedPair = 3,     // two such pairs per block (fewer SMs)
    kPohPairDirect = 4,     // no queue: one pair per 32 consecutive entries (workspace unused)
    kPohAuto = 5,           // kPohPair or kPohSingle (16 x SMs warps), chosen on the device from the counts
};
size_t poh_batch_workspace_size(uint64_t n);
// A served-loop PoH launch that gives way to signature work (kPohPair only):
// every 128 hashes its round warps read the signature service's FIFO and,
// while at least `chunks` published chunks wait unclaimed, sleep (bounded),
// leaving their SM sub-partitions to the service's warps.  A chain's result
// does not depend on when it runs.
struct PohYield {
    const uint32_t* head;    // SvcDevice::head, device memory
    const uint32_t* tail;    // SvcDevice::tail
    uint32_t chunks;         // 0: never
};
cudaError_t launch_poh_batch(uint8_t* hashes, const uint64_t* counts, uint64_t n, void* workspace, int warps,
                             cudaStream_t s, int form = kPohSingle, const PohYield* yield = nullptr);
// The direct paired form alone: poh_pair_persistent_kernel without a queue,
// one block of two warps per 32 consecutive entries.
cudaError_t launch_poh_pair_direct(uint8_t* hashes, const uint64_t* counts, uint64_t n, cudaStream_t s);

// Mixed verify + sign work for one persistent launch (sig_batch.cu).  Both
// batches index the same packet buffer.  Verify items are chunks
// [0, ceil(v.n / 32)); sign items start at chunk sign_base / 32.
struct SigWork {
    SigBatch v;              // out = v.n verdict bytes
    SigBatch s;              // out = s.n * 64 signature bytes
    uint32_t sign_base;      // first sign item's queue position (multiple of 32)
    uint32_t total_chunks;   // chunks of 32 items
    uint32_t* next;          // queue head, device word (reset by the launch)
    // Verify-only launches whose item count is produced on the device: the
    // kernel verifies *count_dev items (v.n and total_chunks are then the
    // capacity, used only to size the grid).
    const uint32_t* count_dev = nullptr;
    // Set by launch_sig_batch: verify chunks of 8 signatures, four lanes each
    // (small batches); otherwise chunks of 32, one lane each.
    bool v_quad = false;
    // Set by launch_sig_batch for count_dev launches: the kernel takes the
    // four-lane form when *count_dev <= v_quad_max (0: never by count).
    uint32_t v_quad_max = 0;
    // Caller's choice: -1 by batch size, kVerifySingle / kVerifyQuad to force.
    int v_form_hint = -1;
};
cudaError_t launch_sig_batch(const SigWork& w, int threads, int blocks_per_sm, int sms, cudaStream_t s);

// Solana ledger entries (poh_entries.cu): PoH chains with transaction
// mixins.  Verification runs every entry's plain hashes as one ragged PoH
// batch, then the mixin step and the comparison; the workspace holds
// poh_entries_workspace_size(n) bytes (256-byte aligned).  Recording runs
// independent chains of entries, one thread per chain.
size_t poh_entries_workspace_size(uint64_t n);
cudaError_t launch_poh_verify_entries(const uint8_t* start, const uint64_t* num_hashes, const uint8_t* mixins,
                                      const uint8_t* has_mixin, const uint8_t* expected, uint64_t n, uint8_t* ok,
                                      uint8_t* out_hashes, void* ws, int warps, cudaStream_t s);
cudaError_t launch_poh_record(uint8_t* hashes, uint64_t chains, const uint64_t* first, uint64_t num_entries,
                              const uint64_t* num_hashes, const uint8_t* mixins, const uint8_t* has_mixin,
                              uint8_t* entry_hashes, cudaStream_t s);
cudaError_t preload_poh_entries_kernels();

// Resident signature service (sig_service.cu) for the served loop: warps of
// one long-lived launch take chunks of signature work from a FIFO in order
// of publication and report each request's completion to the host as soon
// as its last chunk is done.
//   * requests and chunk descriptors live in page-locked host memory the GPU
//     reads (written by the host before the chunks are published);
//   * packets and the per-signature arrays are copied to device memory, and
//     the chunks are published by a stream write of `tail` that follows
//     those copies on the same stream (so a published chunk's inputs are in
//     place);
//   * results go straight into page-locked host memory, then the request's
//     slot in `done` receives its generation number.
struct alignas(16) SvcReq {
    SigBatch b;              // n = the request's items; out: host memory the GPU writes
    uint32_t gen;            // written to done[slot] when the last item is done
    uint32_t pad[3];
};
enum SvcMode : uint32_t { kSvcVerify = 0, kSvcVerifyQuad = 1, kSvcSign = 2 };
struct alignas(16) SvcChunk {
    uint32_t req;            // request slot
    uint32_t first;          // first item
    uint32_t count;          // items: 1..32 (1..8 for kSvcVerifyQuad)
    uint32_t mode;           // SvcMode
};
struct SvcDevice {           // device memory, zeroed at creation
    uint32_t tail;           // chunks published
    uint32_t head;           // chunks claimed
    uint32_t stop;           // nonzero: warps leave as soon as the FIFO is empty
    uint32_t exiting;        // nonzero: the launch is idle and every warp leaves (reset before a launch)
    uint64_t last_claim_ns;  // %globaltimer of the launch's latest claim (reset before a launch)
    uint32_t busy_first;     // preferred warps running a chunk (reset before a launch)
    uint32_t warps;          // warps that started (diagnostic)
    uint32_t sm_blocks[256]; // blocks of the launch started on each SM (reset before a launch)
};
struct SvcParams {
    SvcDevice* dev;
    uint32_t* items_done;    // device memory [max_req], zeroed; each slot returns to 0 on completion
    const SvcReq* req;       // device view of the host request table [max_req]
    const SvcChunk* ring;    // device view of the host chunk ring [ring_size], ring_size a power of two
    uint32_t* done;          // device view of the host completion words [max_req]
    uint64_t* first_claim;   // device memory [max_req], all ones between requests: %globaltimer of a
                             // request's first claimed chunk
    uint64_t* times;         // device view of host memory [2 * max_req]: a completed request's first
                             // claim and completion times (%globaltimer), written before `done`
    uint32_t ring_size;
    uint32_t first_warps;    // warps of the first block on each SM (one per sub-partition), all SMs
    const uint32_t* poh_slots;       // PoH round warps per SM sub-partition (poh_round_warp_map)
    const uint32_t* poh_busy_slots;  // sub-partitions with a PoH round warp
    uint64_t idle_ns;        // the launch leaves (all warps together) after this long without a claim
    const CurveTables* tables;
};
// The L1 / shared-memory split (percent of the largest shared size) that
// the persistent PoH kernels and the resident signature kernel ask for, so
// that neither waits for the other to drain an SM: 164 of 228 KB shared.
// Two service blocks (2 x 60.4 KB) and two PoH pair blocks (2 x 14.3 KB)
// fit, and L1 keeps ~92 KB for the verify path's per-thread point tables
// (local memory).
constexpr int kServeCarveoutPercent = 72;

// SMs covered by the PoH placement map (poh_batch.cu); SM indices wrap.
constexpr uint32_t kMaxServeSms = 256;
// Device addresses of the PoH round warps' placement map on the current
// device: round warps per SM sub-partition (kMaxServeSms x 4) and the count
// of sub-partitions with at least one.
cudaError_t poh_round_warp_map(const uint32_t** per_slot, const uint32_t** busy_slots);

// Blocks of the service kernel that fit on one SM (sets its shared-memory
// attributes on the current device first).
cudaError_t sig_service_blocks_per_sm(int* blocks);
cudaError_t launch_sig_service(const SvcParams& p, int blocks_per_sm, int sms, cudaStream_t s);
// One thread writes %globaltimer to *out (device-visible memory).
cudaError_t launch_svc_clock(uint64_t* out, cudaStream_t s);
cudaError_t preload_sig_service_kernels();

// Solana wire-format packet batches (packets.cu): `n` packet slots `stride`
// bytes apart in one device buffer, lens[i] bytes of transaction data in
// slot i.  The workspace (packets_workspace_size bytes, 256-byte aligned)
// holds the parse results and up to packets_signature_capacity signatures.
size_t packets_workspace_size(uint32_t n, uint64_t stride);
uint64_t packets_signature_capacity(uint32_t n, uint64_t stride);
// The reference's four per-signature arrays (capacity entries each),
// per-packet signature counts (nullable) and the total (device word,
// nullable), all produced on the device.
cudaError_t launch_packets_extract(const uint8_t* data, uint64_t stride, uint32_t n, const uint32_t* lens, void* ws,
                                   size_t ws_bytes, uint32_t* message_lens, uint32_t* key_offsets,
                                   uint32_t* sig_offsets, uint32_t* msg_offsets, uint32_t* counts_out,
                                   uint32_t* total_out, cudaStream_t s);
// Parse, verify every signature, packet_out[i] = 1 iff packet i parsed and
// all its signatures verified; counts_out (nullable) = signatures per packet.
cudaError_t launch_packets_verify(const uint8_t* data, uint64_t stride, uint32_t n, const uint32_t* lens, void* ws,
                                  size_t ws_bytes, uint8_t* packet_out, uint32_t* counts_out,
                                  const CurveTables* tables, int sig_threads, int sig_blocks_per_sm, int sms,
                                  cudaStream_t s, int verify_window = 4);

// Per-device state the served loop (server.cu) needs from the pool
// (crypt_api.cu): device tables and the autotuner's launch shapes.
struct CryptDeviceInfo {
    const CurveTables* tables;
    int sms;
    int sig_threads;
    int sig_blocks_per_sm;
    int verify_window;      // window width of h in the one-lane verify
    int poh_warps;          // resident warps for the persistent PoH kernel
};
bool crypt_device_info(int dev, CryptDeviceInfo* out);
