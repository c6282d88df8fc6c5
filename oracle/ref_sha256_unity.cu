// Test infrastructure only: compiles the reference's LibTomCrypt SHA-256
// (src/cuda-sha256/sha256.cu, built with -DENDIAN_NEUTRAL -DLTC_NO_ASM as
// src/Makefile:34 does) and chains it the way poh_verify_kernel does
// (src/cuda-poh-verify/poh_verify.cu:12-27), on the host.

#include <string.h>
#include <stdint.h>
#include <assert.h>
#include "sha256.cu"

extern "C" void ref_poh_chain(unsigned char* hash32, unsigned long long num_hashes) {
    for (unsigned long long i = 0; i < num_hashes; i++) {
        hash_state st;
        sha256_init(&st);
        sha256_process(&st, hash32, SHA256_BLOCK_SIZE);
        sha256_done(&st, hash32);
    }
}
