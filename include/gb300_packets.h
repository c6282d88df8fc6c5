/*
 * gb300_packets.h -- Solana wire-format packet batches verified end to end
 * on the GPU (no counterpart in the reference, whose ed25519_verify_many
 * takes per-signature offset arrays that its caller computes on the host:
 * src/cuda-ecc-ed25519/verify.cu:240-258, ed25519.h:57-67).
 *
 * A batch is `num_packets` packet slots `stride` bytes apart (the layout of
 * the reference's gpu_Elems runs with message_size = stride) and one data
 * length per packet.  Each packet holds one transaction in the published
 * wire format:
 *   compact-u16 signature count n (n >= 1), n x 64-byte signatures, then the
 *   message: an optional version byte (top bit set; version 0 only), a
 *   3-byte header whose first byte (required signatures) equals n, a
 *   compact-u16 account-key count k >= n, k x 32-byte keys, the rest.
 * Signature i is checked against key i over the message bytes (message start
 * to the end of the packet's data) with the same acceptance rules as
 * ed25519_verify_many.  compact-u16 values are 7-bit little-endian groups,
 * top bit = more follow, at most 3 bytes, no redundant zero group, <= 0xffff.
 * A packet whose data length exceeds the stride or that does not parse is
 * malformed: 0 signatures, verdict 0.
 *
 * Offsets are 32-bit byte offsets into the batch: num_packets * stride must
 * stay below 4 GiB.
 */
#ifndef GB300_CRYPT_PACKETS_H
#define GB300_CRYPT_PACKETS_H

#include <stddef.h>
#include <stdint.h>
#include "ed25519.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Device workspace for the two device entry points below (bytes). */
size_t gb300_packets_workspace_size(uint32_t num_packets, uint64_t stride);

/* Upper bound of the signatures a batch can hold (64 bytes each inside a
 * slot): the capacity of the per-signature arrays. */
uint64_t gb300_packets_signature_capacity(uint32_t num_packets, uint64_t stride);

/* On-device offset extraction: writes the reference's four per-signature
 * arrays (message_lens, public_key_offsets, signature_offsets,
 * message_start_offsets; gb300_packets_signature_capacity entries each, the
 * first *total_signatures used, packet order), signatures per packet
 * (sig_counts, nullable) and the total (one device word, nullable).  All
 * pointers are device memory; workspace 256-byte aligned.  Enqueued on
 * `stream`; returns a cudaError_t. */
int gb300_packets_extract_offsets_device(const uint8_t* packets, uint64_t stride, uint32_t num_packets,
                                         const uint32_t* packet_lens, void* workspace, size_t workspace_bytes,
                                         uint32_t* message_lens, uint32_t* public_key_offsets,
                                         uint32_t* signature_offsets, uint32_t* message_start_offsets,
                                         uint32_t* sig_counts, uint32_t* total_signatures, void* stream);

/* Parse + verify on the device: packet_out[i] = 1 iff packet i parsed and
 * every one of its signatures verified; sig_counts (nullable) as above.
 * Device pointers, enqueued on `stream`; returns a cudaError_t. */
int gb300_ed25519_verify_packets_device(const uint8_t* packets, uint64_t stride, uint32_t num_packets,
                                        const uint32_t* packet_lens, void* workspace, size_t workspace_bytes,
                                        uint8_t* packet_out, uint32_t* sig_counts, void* stream);

/* Host form: the packets of `elems` (num_elems runs of elems[i].num slots,
 * `stride` bytes each, concatenated as ed25519_verify_many does),
 * packet_lens[total packets], packet_out[total packets], sig_counts
 * (nullable).  Synchronous; returns a cudaError_t (outputs zero on error). */
int gb300_ed25519_verify_packets(const gpu_Elems* elems, uint32_t num_elems, uint32_t stride,
                                 const uint32_t* packet_lens, uint8_t* packet_out, uint32_t* sig_counts);

#ifdef __cplusplus
}
#endif

#endif
