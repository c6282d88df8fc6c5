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

/* ---- Solana ledger entries: PoH chains with transaction mixins ---------
 * No counterpart in the reference library: its caller (Solana's ledger-entry
 * verification) runs each entry's plain hashes through poh_verify_many and
 * finishes the entry on the host.  These entry points do the whole entry on
 * the GPU.  From its start hash h (the previous entry's hash) an entry of
 * num_hashes hashes ends at
 *   no mixin (a tick):      h <- SHA-256(h), num_hashes times;
 *   mixin m (32 bytes, the hash of the entry's transactions):
 *                           h <- SHA-256(h), max(num_hashes, 1) - 1 times,
 *                           then h <- SHA-256(h || m).
 * All 32-byte arrays are n * 32 bytes, entry i at offset 32 i. */

/* Device memory the device form of entry verification needs for n entries. */
size_t gb300_poh_entries_workspace_size(uint64_t num_entries);

/* ok[i] = 1 iff entry i, started from start_hashes[i], ends at expected[i]
 * (has_mixin[i] != 0: mixins[i] is its mixin; otherwise mixins[i] is not
 * read); out_hashes[i] (nullable) receives the computed hash.  Device
 * pointers, 32-byte arrays and the workspace 16-byte aligned, counts 8-byte
 * aligned; enqueued on `stream`; returns a cudaError_t.  The plain hashes of
 * all entries run as one ragged persistent PoH batch (longest first). */
int gb300_poh_verify_entries_device(const uint8_t* start_hashes, const uint64_t* num_hashes, const uint8_t* mixins,
                                    const uint8_t* has_mixin, const uint8_t* expected, uint64_t num_entries,
                                    uint8_t* ok, uint8_t* out_hashes, void* workspace, size_t workspace_bytes,
                                    void* stream);

/* Host form of gb300_poh_verify_entries_device (host buffers, synchronous);
 * returns 0, 1 when no GPU is present, or a cudaError_t. */
int gb300_poh_verify_entries(const uint8_t* start_hashes, const uint64_t* num_hashes, const uint8_t* mixins,
                             const uint8_t* has_mixin, const uint8_t* expected, size_t num_entries, uint8_t* ok);

/* Recording: chain c starts from hashes[c] and runs entries first[c] ..
 * first[c + 1] - 1 in order (first has num_chains + 1 elements, first[0] = 0,
 * non-decreasing, first[num_chains] = num_entries); entry e's hash goes to
 * entry_hashes[e] and hashes[c] ends as chain c's last hash.  Entries at or
 * past num_entries are never read.  Entries of one chain are serial, so the
 * GPU records many chains at once, one thread each.  Device pointers
 * (32-byte arrays 16-byte aligned), enqueued on `stream`; returns a
 * cudaError_t. */
int gb300_poh_record_device(uint8_t* hashes, uint64_t num_chains, const uint64_t* first, uint64_t num_entries,
                            const uint64_t* num_hashes, const uint8_t* mixins, const uint8_t* has_mixin,
                            uint8_t* entry_hashes, void* stream);

/* Host form of gb300_poh_record_device (host buffers, synchronous); returns
 * 0, 1 when no GPU is present, or a cudaError_t. */
int gb300_poh_record(uint8_t* hashes, size_t num_chains, const uint64_t* first, const uint64_t* num_hashes,
                     const uint8_t* mixins, const uint8_t* has_mixin, uint8_t* entry_hashes);

#ifdef __cplusplus
}
#endif

#endif
