/*
 * gb300_serve.h -- served request loop of libcuda-crypt.so (no counterpart
 * in the reference, which only has the synchronous one-batch calls).
 *
 * A server owns one GPU (the device current at creation) and a dispatcher
 * thread.  Requests -- an Ed25519 verify or sign job, a batch of Solana
 * wire-format packets, or a PoH batch -- are queued by any thread and
 * admitted as GPU capacity and device memory free up (device memory held by
 * in-flight requests stays below the configured cap).
 *
 * Verify and sign jobs go by default (sig_mode 0) to a resident signature
 * service: the submitting thread stages the job into rings allocated when
 * the server is created and publishes it, in 32-signature chunks (8 when
 * the verifies in flight leave the GPU idle, four lanes each), to the FIFO of
 * one long-lived kernel on a high-priority stream; each job completes as
 * soon as its own chunks are done, whatever else is in flight, and the
 * kernel leaves after 20 ms without work (launched again on demand;
 * GB300_CRYPT_SERVER_IDLE_US changes the wait).  Jobs too large for the
 * rings (1 GiB of device inputs at most, bounded by the memory cap; 256 MiB
 * of pageable packets; 64 MiB of results; 2^18 chunks) take the slot path.
 * With sig_mode 1, and always for wire-format packet batches, requests that
 * arrive while earlier ones are on the GPU are merged into the next
 * persistent launch of a slot (continuous batching) on high-priority
 * streams.  PoH requests run on a low-priority stream so a long chain does
 * not hold up signature work.  Each request's results are exactly those of
 * the corresponding one-call entry point.
 *
 * The caller's buffers must stay valid, and its outputs untouched, until
 * the request is complete.  Page-locked (cuda_host_register) packet buffers
 * are copied to the GPU directly; others go through the server's staging.
 */
#ifndef GB300_CRYPT_SERVE_H
#define GB300_CRYPT_SERVE_H

#include <stddef.h>
#include <stdint.h>
#include "ed25519.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb300_server gb300_server;

typedef struct {
    uint64_t device_memory_cap;      /* bytes in flight on the GPU; 0 = 8 GiB */
    uint32_t sig_slots;              /* concurrent signature launches; 0 = 3 (2 beside
                                        the signature service) */
    uint32_t poh_slots;              /* concurrent PoH launches; 0 = 2 */
    uint32_t max_items_per_launch;   /* signatures merged into one launch; 0 = 65536
                                        (a larger request runs alone) */
    uint32_t sig_mode;               /* verify/sign jobs: 0 = resident signature service,
                                        1 = merged launches on the slots */
} gb300_server_config;

/* Creates a server on the current device (cfg may be NULL); NULL on failure. */
gb300_server* gb300_server_create(const gb300_server_config* cfg);

/* Finishes every admitted and queued request, then stops. */
void gb300_server_destroy(gb300_server* s);

/* Queues one verify (job->kind 0) or sign (kind 1) job; returns a ticket
 * (> 0) or 0 when the job is invalid or alone exceeds the memory cap. */
uint64_t gb300_server_submit_sigs(gb300_server* s, const gb300_sig_job* job);

/* Queues a batch of Solana wire-format packets, as
 * gb300_ed25519_verify_packets (gb300_packets.h) takes it: num_elems runs of
 * elems[i].num packet slots `stride` bytes apart, packet_lens[total packets];
 * on completion packet_out[i] = 1 iff packet i parsed and all its signatures
 * verified, sig_counts[i] (nullable) = its signatures.  The descriptors in
 * `elems` are copied; the packet data, lengths and outputs must stay valid
 * until completion.  Batches of one stride merge into one launch that parses
 * on the GPU.  Ticket, or 0 when the batch is invalid (no packets, null
 * pointers, total slot bytes of 4 GiB or more) or alone exceeds the memory
 * cap. */
uint64_t gb300_server_submit_packets(gb300_server* s, const gpu_Elems* elems, uint32_t num_elems, uint32_t stride,
                                     const uint32_t* packet_lens, uint8_t* packet_out, uint32_t* sig_counts);

/* Queues a PoH batch (in place on hashes, as poh_verify_many); ticket or 0. */
uint64_t gb300_server_submit_poh(gb300_server* s, uint8_t* hashes, const uint64_t* num_hashes, size_t num_elems);

/* 1 when the request is complete, 0 while pending, negative cudaError_t on
 * failure (the outputs are then zero). */
int gb300_server_poll(gb300_server* s, uint64_t ticket);

/* Blocks until completion or timeout_ms (< 0: no limit); returns as poll. */
int gb300_server_wait(gb300_server* s, uint64_t ticket, int timeout_ms);

/* Forgets a completed ticket (frees its bookkeeping). */
void gb300_server_release(gb300_server* s, uint64_t ticket);

/* Submission and completion times of a ticket (steady clock, ns; done_ns
 * is -1 while pending); returns 1 when complete, 0 while pending. */
int gb300_server_times(gb300_server* s, uint64_t ticket, int64_t* submit_ns, int64_t* done_ns);

/* Timeline of the most recent launches as a JSON array of
 * [kind (0 signatures, 2 PoH, 3 wire packets), requests merged, items,
 *  admitted_ns, enqueued_ns, completed_ns, copy_in_ms, kernels_ms,
 *  copy_out_ms]: host times of the launch, then the GPU time of its input
 * copies, its kernels and its result copy (CUDA events; -1 after a
 * failure).  A job served by the resident signature service appears as
 * [4, 1, items, submitted_ns, published_ns, completed_ns, wait_ms, run_ms,
 * total_ms]: ms from its publication to the GPU's first claim of one of its
 * chunks, from that claim to its completion on the GPU (GPU clock, related
 * to the host clock at server creation; -1 after a failure), and from
 * publication to completion as the host saw it.  Returns the length
 * written. */
int gb300_server_trace(gb300_server* s, char* buf, size_t len);

/* Counters as a JSON object; returns the length written. */
int gb300_server_stats(gb300_server* s, char* buf, size_t len);

#ifdef __cplusplus
}
#endif

#endif
