// Device-resident curve constants and basepoint tables.
//
// Replaces the reference's compile-time tables (src/cuda-ecc-ed25519/
// precomp_data.h: Bi[8] :1, odd multiples of B for verify; base[32][8]
// :45-46, for signing) and the constants d / sqrt(-1) in ge.cu.  Nothing is
// copied: init kernels derive every entry from the curve definition
// (d = -121665/121666, B = (x, 4/5) with x even) when a device is first used.
//
// Layouts, chosen for how the kernels read them:
//   vb  verify table, k*B for k = 0..128 as affine (y+x, y-x, 2dxy), stored
//       word-major ("structure of arrays": word w of entry k at
//       vb[w * VB_ENTRIES + k]) so that a warp gathering 32 different
//       entries from shared memory hits 32 different banks.
//   comb signing table, (j+1) * 16^i * B for i = 0..63, j = 0..7, affine,
//       entry-major; a warp reads all 8 entries of one window together
//       (constant-time select), i.e. broadcast reads.
#pragma once
#include "ge25519.cuh"

#define VB_ENTRIES 129          // 0..128
#define VB_WORDS 24             // 3 field elements
#define COMB_WINDOWS 64
#define COMB_ENTRIES 8

struct CurveTables {
    CurveConsts K;
    fe B_x, B_y;
    uint32_t vb[VB_WORDS * VB_ENTRIES];
    ge_niels comb[COMB_WINDOWS][COMB_ENTRIES];
};

#ifdef __cplusplus
// Creates (once per device) the tables on the current device; returns a
// device pointer or nullptr on failure.  Defined in tables.cu.
cudaError_t crypt_tables_create(CurveTables** out, cudaStream_t stream);
#endif
