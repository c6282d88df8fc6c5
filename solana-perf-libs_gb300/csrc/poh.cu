// Proof-of-History chain verification kernels.
//
// Replaces the reference's poh_verify_kernel (src/cuda-poh-verify/
// poh_verify.cu:12-27): one thread per entry, hash <- SHA-256(hash)
// num_hashes[i] times, in place.  The chain state lives in eight registers
// for the whole chain; the 32-byte entries are read and written as two
// 16-byte vectors.
#include <cuda_runtime.h>
#include "kernels.h"
#include "sha256_poh.cuh"

// One warp per block: 4096 entries then spread over 128 SMs, one warp on a
// sub-partition each (measured 4.5% faster than two warps per SM).  A chain
// is a serial dependency, so a warp is bound by its sub-partition's ALU pipe
// (16 lanes/clock); fewer active lanes per warp do not change that.
#ifndef POH_THREADS
#define POH_THREADS 32
#endif
// How many rotations of Sigma0 / Sigma1 / each schedule sigma run on the
// multiply pipe (see poh_step_mix).
// POH_NO_PAIR=1 disables the two-warp kernel (measurement switch).
#ifndef POH_NO_PAIR
#define POH_NO_PAIR 0
#endif
#ifndef POH_NS0
#define POH_NS0 0
#endif
#ifndef POH_NS1
#define POH_NS1 0
#endif
#ifndef POH_NSG
#define POH_NSG 0
#endif

namespace {

__device__ __forceinline__ uint32_t bswap(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

__device__ __forceinline__ void poh_chain(uint8_t* entry, uint64_t count, uint32_t one) {
    uint4* p = reinterpret_cast<uint4*>(entry);
    uint4 lo = p[0], hi = p[1];
    uint32_t w[8] = {bswap(lo.x), bswap(lo.y), bswap(lo.z), bswap(lo.w),
                     bswap(hi.x), bswap(hi.y), bswap(hi.z), bswap(hi.w)};
    const PohMul M(one);
#pragma unroll 1
    for (uint64_t k = 0; k < count; k++) poh_step_mix<POH_NS0, POH_NS1, POH_NSG>(w, M);
    p[0] = make_uint4(bswap(w[0]), bswap(w[1]), bswap(w[2]), bswap(w[3]));
    p[1] = make_uint4(bswap(w[4]), bswap(w[5]), bswap(w[6]), bswap(w[7]));
}

// `one` is always 1; it arrives as a kernel argument so that the rotation
// multipliers derived from it stay opaque to the compiler (see rotr_mul).
__global__ void __launch_bounds__(POH_THREADS) poh_verify_kernel(uint8_t* hashes, const uint64_t* num_hashes,
                                                                 uint64_t n, uint32_t one) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    poh_chain(hashes + 32 * i, num_hashes[i], one);
}

}  // namespace

cudaError_t preload_poh_kernels() { return load_kernels(poh_verify_kernel); }

cudaError_t launch_poh_verify(uint8_t* hashes, const uint64_t* num_hashes, uint64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        return cudaGetLastError();
    // Two warps per 32 chains while the pairs fit one warp per sub-partition.
    // A lone warp is bound by its sub-partition's ALU pipe (one warp
    // instruction every 2 cycles, ~1,330 per hash), and a batch of a few
    // thousand chains leaves most sub-partitions idle: in the paired form
    // (poh_batch.cu) one warp computes the message schedule into shared
    // memory while the other runs the 64 rounds, ~840 instructions per hash
    // on the round warp.
    const uint64_t groups = (n + 31) / 32;
    if (!POH_NO_PAIR && 2 * groups <= 4ull * (uint64_t)sms) return launch_poh_pair_direct(hashes, num_hashes, n, s);
    uint64_t blocks = (n + POH_THREADS - 1) / POH_THREADS;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidValue;
    poh_verify_kernel<<<(unsigned)blocks, POH_THREADS, 0, s>>>(hashes, num_hashes, n, 1u);
    return cudaGetLastError();
}
