// Test infrastructure only: a unity translation unit that compiles the
// reference's own host-callable Ed25519 and SHA-256 code straight from the
// reference tree (the include path is supplied by oracle/ref.mk) so that the
// C restatement in oracle/crypt_oracle.c can be checked against the real
// thing.  Nothing here is shipped or measured.
//
// Exported (C ABI), all host-only:
//   ed25519_verify / ed25519_sign / ed25519_create_keypair /
//   ed25519_get_checked_scalar / ed25519_check_packed_ge_small_order
//     -- the reference's own symbols (src/cuda-ecc-ed25519/ed25519.h:25-81)
//   ref_sc_reduce, ref_sc_muladd, ref_scalarmult_base, ref_poh_chain
//     -- thin wrappers over reference internals (sc.cu:238, sc.cu:565,
//        ge.cu:452, sha256.cu:198-277) for piecewise pinning.

#include "verify.cu"
#include "sign.cu"
#include "keypair.cu"
#include "gpu_ctx.cu"

extern "C" void ref_sc_reduce(unsigned char* s64) { sc_reduce(s64); }

extern "C" void ref_sc_muladd(unsigned char* s, const unsigned char* a,
                              const unsigned char* b, const unsigned char* c) {
    sc_muladd(s, a, b, c);
}

extern "C" void ref_scalarmult_base(unsigned char* out32, const unsigned char* a32) {
    ge_p3 A;
    ge_scalarmult_base(&A, a32);
    ge_p3_tobytes(out32, &A);
}

// R' = a*A' + b*B where A' is the (negated) decode of A; returns 0 if A does
// not decode.  Mirrors the reference's verify data flow without the checks.
extern "C" int ref_double_scalarmult(unsigned char* out32, const unsigned char* a32,
                                     const unsigned char* A32, const unsigned char* b32) {
    ge_cached Ai[GE_LOOKUP_SIZE];
    ge_p3 A;
    if (0 != ge_frombytes_negate_vartime(&A, A32)) return 0;
    ge_p1p1 t;
    ge_p3 u;
    ge_p3 A2;
    ge_p3_to_cached(&Ai[0], &A);
    ge_p3_dbl(&t, &A);
    ge_p1p1_to_p3(&A2, &t);
    for (int k = 1; k < GE_LOOKUP_SIZE; k++) {
        ge_add(&t, &A2, &Ai[k - 1]);
        ge_p1p1_to_p3(&u, &t);
        ge_p3_to_cached(&Ai[k], &u);
    }
    ge_p2 R;
    ge_double_scalarmult_vartime(&R, a32, Ai, b32);
    ge_tobytes(out32, &R);
    return 1;
}
