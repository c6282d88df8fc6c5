/*
 * gb300_diag.h -- diagnostics of libcuda-crypt.so (no counterpart in the
 * reference): integer-pipe throughput microbenchmarks used as the
 * denominators of the integer roofline that the benchmark reports.
 */
#ifndef GB300_CRYPT_DIAG_H
#define GB300_CRYPT_DIAG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Launches blocks x threads (threads <= 256) threads, each running iters
 * rounds of 16 dependent-chain ops of one form:
 *   kind 0 lop3.b32, 1 mad.wide.u32, 2 mad.lo.u32, 3 shf.r.wrap.b32.
 * Executed ops = blocks * threads * iters * 16.  `sink` is a device word
 * the kernel may write.  Enqueued on `stream`; returns a cudaError_t. */
int gb300_int_peak_launch(int kind, uint32_t blocks, uint32_t threads, uint32_t iters, uint32_t* sink,
                          void* stream);

#ifdef __cplusplus
}
#endif

#endif
