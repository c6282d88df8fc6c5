/*
 * gb300_diag.h -- diagnostics of libcuda-crypt.so (no counterpart in the
 * reference): integer-pipe throughput microbenchmarks used as the
 * denominators of the integer roofline that the benchmark reports, and a
 * PoH batch entry point with a forced launch shape.
 */
#ifndef GB300_CRYPT_DIAG_H
#define GB300_CRYPT_DIAG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Launches blocks x threads (threads <= 256) threads, each running iters
 * rounds of 16 dependent-chain ops of one form:
 *   kind 0 lop3.b32, 1 mad.wide.u32, 2 mad.lo.u32, 3 shf.r.wrap.b32,
 *   4 the SHA-256 proportions: 8 lop3.b32 + 4 shf.r.wrap.b32 + 4 mad.lo.u32
 *   per 16, 5 the fastest measured mix: 4 lop3.b32 + 4 shf.r.wrap.b32 +
 *   8 add.u32 per 16.
 * Executed ops = blocks * threads * iters * 16.  `sink` is a device word
 * the kernel may write.  Enqueued on `stream`; returns a cudaError_t. */
int gb300_int_peak_launch(int kind, uint32_t blocks, uint32_t threads, uint32_t iters, uint32_t* sink,
                          void* stream);

/* gb300_poh_verify_batch_device with the launch shape forced instead of
 * tuned: `warps` resident warps (1 .. 64 x SM count; a pair counts two) of
 * the persistent kernel in form
 *   0  one warp per 32 chains, one warp per block
 *   1  one warp per 32 chains, four warps per block
 *   2  a schedule warp and a round warp per 32 chains, one pair per block
 *   3  two such pairs per block
 *   4  no queue: one pair per 32 consecutive entries (`warps` unused)
 *   5  form 2 with `warps`, or form 0 with 16 x SM count warps, chosen on the
 *      device from the longest count and the sum of the counts.
 * Same results as every other PoH entry point; used to test and time each
 * form.  Returns a cudaError_t. */
int gb300_poh_verify_batch_shape(uint8_t* hashes, const uint64_t* num_hashes, uint64_t num_elems, void* workspace,
                                 size_t workspace_bytes, int warps, int form, void* stream);

/* gb300_ed25519_verify_device with the kernel form forced instead of picked
 * by batch size: form 0 one thread per signature (the tuned window width of
 * h), 1 four lanes per signature, 2 one thread per signature with a 4-bit
 * window, 3 the same with a 5-bit window, 4 three warps per eight
 * signatures with half-size scalars, 5 one thread per signature (4-bit
 * window) with the signatures and keys staged through shared memory by
 * coalesced 16-byte loads, 6 one thread per signature with half-size
 * scalars (form 0 is the autotuner's choice of 6 or 2).  Same verdicts in every form; used to test and
 * time each.  Returns a cudaError_t. */
int gb300_ed25519_verify_device_form(const uint8_t* packets, uint64_t packets_len, const uint32_t* message_lens,
                                     const uint32_t* public_key_offsets, const uint32_t* signature_offsets,
                                     const uint32_t* message_start_offsets, uint32_t num, uint8_t* out, int form,
                                     void* stream);

/* The half-size scalars the three-warp verify form uses: for each of `num`
 * values h < L (8 little-endian 32-bit words each, device memory) writes 18
 * words to `out` (device memory): |c| (8 words), all ones when c < 0 else 0,
 * d (8 words), and the rounds of the lattice reduction; c = d h (mod 8L)
 * with d odd and positive, (c, d) = (h, 1) when no short pair fits.  Used
 * to test the reduction on chosen h.  Returns a cudaError_t. */
int gb300_diag_half_scalars(const uint32_t* h, uint32_t num, uint32_t* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif
