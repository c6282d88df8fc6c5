/*
 * ed25519.h -- C ABI of libcuda-crypt.so, the GB300 build of the
 * solana-perf-libs hot path (batched Ed25519 verify/sign and SHA-256
 * Proof-of-History verification).
 *
 * Every entry point in the first part has the name, argument list and
 * meaning of the reference's export it replaces (paths inside the reference
 * tree; the exported symbol set of its libcuda-crypt.so), so a loader that
 * binds the reference library (solana_perf::perf_libs) binds this one.
 * Differences in error behaviour are stated per function.
 *
 * All computation runs on the GPU; functions return after their results are
 * in the caller's buffers.  Thread-safe: calls are spread round-robin over
 * up to 8 GPUs, then to the first idle of 8 queues on that GPU, each queue
 * serialised by its own lock.
 */
#ifndef GB300_CRYPT_ED25519_H
#define GB300_CRYPT_ED25519_H

#include <stddef.h>
#include <stdint.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SHA512_SIZE 64
#define PUB_KEY_SIZE 32
#define PRIV_KEY_SIZE 64
#define SEED_SIZE 32
#define SCALAR_SIZE 32
#define SIG_SIZE 64

/* A run of num packets, each message_size bytes (the packet stride), stored
 * back to back; batches are concatenated in order and all offsets are byte
 * offsets into that concatenation.  Reference: src/cuda-ecc-ed25519/ed25519.h:35-38. */
typedef struct {
    uint8_t* elems;
    uint32_t num;
} gpu_Elems;

/* Creates the GPU contexts and device tables.  false when no GPU is usable.
 * Reference: ed25519.h:74, gpu_ctx.cu:38-44. */
bool ed25519_init(void);

/* Verbose logging on stdout.  Reference: ed25519.h:71, verify.cu:236. */
void ed25519_set_verbose(bool val);

/* Verifies total_signatures signatures; out[i] = 1 (valid) or 0.
 * signature i: 64 bytes at signature_offsets[i], public key 32 bytes at
 * public_key_offsets[i], message message_lens[i] bytes at
 * message_start_offsets[i].  Acceptance is bit-exact with the reference,
 * quirks included (S with any of its top 4 bits set is rejected; R or A of
 * order dividing 4 is rejected, order 8 is not; y >= p is accepted on
 * decode).  total_packets == 0 or total_signatures == 0: returns, out
 * untouched.  Differences: an offset/length that reaches past the packet
 * data gives verdict 0 (the reference reads out of bounds); a CUDA failure
 * gives all-zero verdicts and sets gb300_crypt_last_error() (the reference
 * aborts).  Reference: ed25519.h:57-67, verify.cu:240-340. */
void ed25519_verify_many(const gpu_Elems* elems, uint32_t num_elems, uint32_t message_size,
                         uint32_t total_packets, uint32_t total_signatures, const uint32_t* message_lens,
                         const uint32_t* public_key_offsets, const uint32_t* signature_offsets,
                         const uint32_t* message_start_offsets, uint8_t* out, uint8_t use_non_default_stream);

/* Signs total_signatures messages; signatures_out[64*i..] = R || S,
 * byte-identical to the reference.  The 64-byte private key of item i
 * (clamped scalar || nonce prefix, as ed25519_create_keypair makes it) is at
 * private_key_offsets[i].  Out-of-range offsets give an all-zero signature.
 * Reference: ed25519.h:43-53, sign.cu:76-145. */
void ed25519_sign_many(const gpu_Elems* elems, uint32_t num_elems, uint32_t message_size,
                       uint32_t total_packets, uint32_t total_signatures, const uint32_t* message_lens,
                       const uint32_t* public_key_offsets, const uint32_t* private_key_offsets,
                       const uint32_t* message_start_offsets, uint8_t* signatures_out,
                       uint8_t use_non_default_stream);

/* Single-item forms (run on the GPU as batches of one).
 * Reference: ed25519.h:25,40,41,55; keypair.cu:6-16; sign.cu:40-46; verify.cu:154-174. */
int ed25519_create_seed(unsigned char* seed);
void ed25519_create_keypair(unsigned char* public_key, unsigned char* private_key, const unsigned char* seed);
void ed25519_sign(unsigned char* signature, const unsigned char* message, size_t message_len,
                  const unsigned char* public_key, const unsigned char* private_key);
int ed25519_verify(const unsigned char* signature, const unsigned char* message, uint32_t message_len,
                   const unsigned char* public_key);

/* 0 when S (32 bytes) is accepted by the verifier (top 4 bits clear), and
 * then out_scalar = in_scalar.  Reference: ed25519.h:79, verify.cu:60-85. */
int ed25519_get_checked_scalar(unsigned char* out_scalar, const unsigned char* in_scalar);

/* 0 when the 32-byte encoding decodes and its point's order does not
 * divide 4.  Reference: ed25519.h:81, verify.cu:88-107. */
int ed25519_check_packed_ge_small_order(const unsigned char* packed_group_element);

/* Page-locks / unlocks caller memory (returns the raw cudaError_t).
 * Reference: ed25519.h:76-77, verify.cu:349-355. */
int cuda_host_register(void* ptr, size_t size, unsigned int flags);
int cuda_host_unregister(void* ptr);

/* Reference: ed25519.h:73 (license string), gpu_ctx.h:39 (frees the pooled
 * device buffers; the next call re-grows them). */
const char* ed25519_license(void);
void ed25519_free_gpu_mem(void);

/* ---- additions of this library (no counterpart in the reference) ------- */

/* cudaError_t of the last failed call on this thread (0 = none); cleared by
 * every successful call. */
int gb300_crypt_last_error(void);

/* Device-pointer forms: same work on buffers already resident in GPU memory,
 * enqueued on `stream` (a cudaStream_t, 0 = legacy default stream) without
 * synchronising.  Buffers must be 4-byte aligned (PoH hashes 16-byte).
 * Return a cudaError_t (0 = launched). */
int gb300_ed25519_verify_device(const uint8_t* packets, uint64_t packets_len, const uint32_t* message_lens,
                                const uint32_t* public_key_offsets, const uint32_t* signature_offsets,
                                const uint32_t* message_start_offsets, uint32_t num, uint8_t* out,
                                void* stream);
int gb300_ed25519_sign_device(const uint8_t* packets, uint64_t packets_len, const uint32_t* message_lens,
                              const uint32_t* public_key_offsets, const uint32_t* private_key_offsets,
                              const uint32_t* message_start_offsets, uint32_t num, uint8_t* signatures_out,
                              void* stream);
int gb300_ed25519_keypair_device(const uint8_t* seeds, uint8_t* public_keys, uint8_t* private_keys, uint32_t num,
                                 void* stream);

/* Batched keypair generation on host buffers (32-byte seeds -> 32-byte
 * public keys, 64-byte private keys); returns a cudaError_t. */
int gb300_ed25519_create_keypairs(const uint8_t* seeds, uint8_t* public_keys, uint8_t* private_keys,
                                  uint32_t num);

/* One job of a ragged batch: a packet buffer with the reference's
 * per-signature arrays (offsets relative to this job's packets).  kind 0
 * verifies (key_offsets = signature offsets, out = num verdict bytes),
 * kind 1 signs (key_offsets = 64-byte private key offsets, out = 64*num
 * signature bytes). */
typedef struct {
    const uint8_t* packets;
    uint64_t packets_len;
    const uint32_t* message_lens;
    const uint32_t* public_key_offsets;
    const uint32_t* key_offsets;
    const uint32_t* message_start_offsets;
    uint32_t num;
    uint32_t kind;
    uint8_t* out;
} gb300_sig_job;

/* Runs every job in ONE persistent launch (verify chunks first, then sign
 * chunks, pulled from a device queue by a resident grid whose shape the
 * autotuner picked), replayed from a captured CUDA graph when the batch
 * shape repeats.  Results are exactly those of ed25519_verify_many /
 * ed25519_sign_many on each job.  Total packet bytes must stay below 4 GiB.
 * Returns a cudaError_t. */
int gb300_ed25519_batch(const gb300_sig_job* jobs, uint32_t num_jobs);

/* Device-pointer form of one mixed batch: nv verify items and ns sign items
 * over one device packet buffer; `queue_word` is one device uint32 the
 * launch uses as its queue head.  Enqueued on `stream`. */
int gb300_ed25519_batch_device(const uint8_t* packets, uint64_t packets_len,
                               const uint32_t* v_message_lens, const uint32_t* v_public_key_offsets,
                               const uint32_t* v_signature_offsets, const uint32_t* v_message_start_offsets,
                               uint32_t nv, uint8_t* v_out,
                               const uint32_t* s_message_lens, const uint32_t* s_public_key_offsets,
                               const uint32_t* s_private_key_offsets, const uint32_t* s_message_start_offsets,
                               uint32_t ns, uint8_t* s_out, uint32_t* queue_word, void* stream);

/* The autotuner's choices for the current GPU as a JSON object (runs the
 * tuner on first use); returns the length written (truncated to len - 1). */
int gb300_crypt_tuning(char* buf, size_t len);

#ifdef __cplusplus
}
#endif

#endif
