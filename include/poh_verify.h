/*
 * poh_verify.h -- Proof-of-History chain verification in libcuda-crypt.so.
 *
 * Reference: src/cuda-poh-verify/poh_verify.cu:74-145 (the reference
 * declares these in that .cu file only; the symbols are exported from its
 * libcuda-crypt.so).
 */
#ifndef GB300_CRYPT_POH_VERIFY_H
#define GB300_CRYPT_POH_VERIFY_H

#include <stddef.h>
#include <stdint.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

/* hashes[32*i .. 32*i+32) <- SHA-256 applied num_hashes_arr[i] times, in
 * place (num_hashes_arr[i] == 0 leaves the entry unchanged).  Returns 0 on
 * success, 1 when no GPU is present (as the reference), and the cudaError_t
 * of a failed CUDA call otherwise (the reference aborts).  The caller
 * compares the results with its expected hashes; there is no pass/fail
 * output.  Reference: poh_verify.cu:80-144. */
int poh_verify_many(uint8_t* hashes, const uint64_t* num_hashes_arr, size_t num_elems,
                    uint8_t use_non_default_stream);

/* Reference: poh_verify.cu:76. */
void poh_verify_many_set_verbose(bool val);

/* ---- additions of this library (no counterpart in the reference) ------- */

/* Device-pointer form: hashes (16-byte aligned) and counts already in GPU
 * memory, enqueued on `stream` without synchronising; returns a cudaError_t. */
int gb300_poh_verify_device(uint8_t* hashes, const uint64_t* num_hashes, uint64_t num_elems, void* stream);

/* Ragged batches: same results as poh_verify_many, computed by one
 * persistent launch that orders entries longest first (by bit length of the
 * count) and keeps every lane busy by refilling it from a device queue;
 * replayed from a captured CUDA graph when the batch shape repeats.
 * Returns 0 or a cudaError_t. */
int gb300_poh_verify_batch(uint8_t* hashes, const uint64_t* num_hashes_arr, size_t num_elems);

/* Device-memory scratch the device form needs for num_elems entries. */
size_t gb300_poh_batch_workspace_size(uint64_t num_elems);

/* Device form: hashes (16-byte aligned), counts and workspace (at least
 * gb300_poh_batch_workspace_size bytes, 16-byte aligned) in GPU memory;
 * enqueued on `stream`.  The launch shape (a schedule and a round warp per
 * 32 chains, or one warp per 32 chains) is chosen on the GPU from the
 * longest count and the sum of the counts, as gb300_poh_verify_batch
 * chooses it on the host. */
int gb300_poh_verify_batch_device(uint8_t* hashes, const uint64_t* num_hashes, uint64_t num_elems,
                                  void* workspace, size_t workspace_bytes, void* stream);

/* Same work as gb300_poh_verify_batch_device without a workspace argument
 * and without allocating anything.  No counterpart in the reference.  It is
 * for callers that may not call cudaMalloc (GPU memory owned by a pooling
 * allocator with a fixed budget, or a pipeline that must not take the
 * device-wide synchronisation cudaMalloc/cudaFree can cause): its scratch is
 * a 1 MiB array built into the library, so at most 262,144 entries per call
 * (more returns cudaErrorInvalidValue with a message on stderr).  The first
 * call on each device looks up that array's device address; make that first
 * call before any stream capture.  The address is kept for the life of the
 * process and belongs to the device's primary context (the one the CUDA
 * runtime uses): do not call it from another context, nor after
 * cudaDeviceReset.  All calls share the one array, so calls
 * that overlap on the GPU (concurrent streams or threads) race: serialise
 * them.  hashes 16-byte and counts 8-byte aligned; enqueued on `stream`;
 * returns 0 or a cudaError_t. */
int gb300_poh_verify_batch_static(uint8_t* hashes, const uint64_t* num_hashes, uint64_t num_elems, void* stream);

#ifdef __cplusplus
}
#endif

#endif
