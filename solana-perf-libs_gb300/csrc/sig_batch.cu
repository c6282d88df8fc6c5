// Ragged Ed25519 batches: many verify and sign jobs in one persistent launch.
//
// The reference's drop-in entry points (and ours, verify.cu / sign.cu) take
// one batch per call: one launch, one copy each way, one synchronisation, and
// a grid sized to that batch, so a small batch leaves most SMs idle while
// the host pays the fixed cost per call.  Here all jobs are concatenated:
//   * items are split into chunks of 32 (one warp); verify chunks come first
//     (a verification costs about four signings: longest first), sign chunks
//     start at the next multiple of 32;
//   * a persistent grid (blocks resident on every SM, threads per block and
//     blocks per SM chosen by the autotuner) pulls chunks from a queue head
//     in device memory until the queue is empty, so a warp that drew cheap
//     chunks (early rejections, short messages) simply takes more;
//   * each block stages the verify basepoint table into shared memory once.
#include <cuda_runtime.h>
#include <atomic>
#include <cstdlib>
#include "kernels.h"
#include "tables.cuh"
#include "sha512.cuh"
#include "sc25519.cuh"

namespace {

#include "ed25519_ops.cuh"
#include "verify_quad.cuh"

// Chunk counts of a launch: verify chunks (32 signatures, or 8 in quad
// mode), then sign chunks of 32.
__host__ __device__ __forceinline__ uint32_t verify_chunks(const SigWork& w, uint32_t vn, bool quad) {
    if (quad) return (vn + 7u) / 8u;
    return w.count_dev ? (vn + 31u) / 32u : w.sign_base / 32u;
}
__host__ __device__ __forceinline__ uint32_t sign_chunks(const SigWork& w) {
    return w.count_dev ? 0u : w.total_chunks - w.sign_base / 32u;
}

// Launches with sign items also stage the signing comb (48 KB) into dynamic
// shared memory: each sign reads all 8 entries of 64 windows, and from
// global memory those reads stall on the L1 round trip.
constexpr size_t kCombBytes = sizeof(ge_niels) * COMB_WINDOWS * COMB_ENTRIES;

// MINB > 0: the build capped for MINB blocks per SM (more warps to hide the
// dependent carry chains, some spills), used for launches that fill them.
template <int T, int W, int MINB>
__global__ void __launch_bounds__(T, MINB) sig_persistent_kernel(SigWork w) {
    __shared__ uint32_t sVB[VB_WORDS * VB_ENTRIES];
    extern __shared__ uint4 s_comb4[];
    for (int k = threadIdx.x; k < VB_WORDS * VB_ENTRIES; k += blockDim.x) sVB[k] = w.v.tables->vb[k];
    const bool comb_in_smem = w.s.n > 0;          // launch-uniform: dynamic size is kCombBytes then
    if (comb_in_smem) {
        const uint4* g = reinterpret_cast<const uint4*>(&w.s.tables->comb[0][0]);
        for (uint32_t k = threadIdx.x; k < kCombBytes / 16; k += blockDim.x) s_comb4[k] = g[k];
    }
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t vn = w.count_dev ? *w.count_dev : w.v.n;
    const bool quad = w.v_quad || (w.v_quad_max && vn <= w.v_quad_max);   // launch-uniform
    const uint32_t vchunks = verify_chunks(w, vn, quad);
    const uint32_t chunks = vchunks + sign_chunks(w);
    for (;;) {
        uint32_t c = 0;
        if (lane == 0) c = atomicAdd(w.next, 1u);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= chunks) break;
        if (c < vchunks) {
            if (quad) {
                // every lane runs an item (past the end: the last one again,
                // result dropped) so the whole warp meets every shuffle
                const uint32_t i = c * 8u + (lane >> 2);
                const bool ok = verify_quad(w.v, sVB, i < vn ? i : vn - 1u, lane & 3u);
                if (i < vn && (lane & 3u) == 0) w.v.out[i] = ok ? 1 : 0;
            } else {
                // every lane runs an item (past the end: the last one
                // again, result dropped): the half-size-scalar form votes
                // over the warp
                const uint32_t i = c * 32u + lane;
                const bool ok = verify_window<W>(w.v, sVB, i < vn ? i : vn - 1u);
                if (i < vn) w.v.out[i] = ok ? 1 : 0;
            }
        } else {
            const uint32_t i = (c - vchunks) * 32u + lane;
            if (i < w.s.n) sign_one_tab(w.s, i, reinterpret_cast<const ge_niels*>(s_comb4));
        }
    }
}

template <int T, int W, int MINB>
cudaError_t launch_t(const SigWork& w, int blocks_per_sm, int sms, cudaStream_t s) {
    // 12 KB static + 48 KB dynamic shared memory is above the 48 KB a block
    // gets without opting in; the opt-in is an attribute of the function on
    // each device, set on the device's first launch
    static std::atomic<uint64_t> opted{0};      // bit d: done on device d
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = 1ull << (dev & 63);
    if (!(opted.load() & bit)) {
        e = cudaFuncSetAttribute(sig_persistent_kernel<T, W, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kCombBytes);
        if (e != cudaSuccess) return e;
        opted.fetch_or(bit);
    }
    const size_t dyn = w.s.n > 0 ? kCombBytes : 0;
    // resident blocks per SM, per device and with or without the comb: the
    // occupancy query costs host time on every launch otherwise
    static std::atomic<int> occ[64][2];
    std::atomic<int>& slot = occ[dev & 63][dyn ? 1 : 0];
    int maxb = slot.load();
    if (maxb == 0) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, sig_persistent_kernel<T, W, MINB>, T, dyn);
        if (e != cudaSuccess) return e;
        if (maxb < 1) maxb = 1;
        slot.store(maxb);
    }
    int b = blocks_per_sm < 1 ? maxb : (blocks_per_sm < maxb ? blocks_per_sm : maxb);
    // (a launch that may take the four-lane form by its device count is
    // sized for it)
    uint32_t warps_needed = verify_chunks(w, w.v.n, w.v_quad || w.v_quad_max > 0) + sign_chunks(w);
    uint32_t grid = (uint32_t)(b * sms);
    uint32_t per_block = T / 32;
    if (grid * per_block > warps_needed) grid = (warps_needed + per_block - 1) / per_block;
    if (grid == 0) return cudaSuccess;
    sig_persistent_kernel<T, W, MINB><<<grid, T, dyn, s>>>(w);
    return cudaGetLastError();
}

}  // namespace

cudaError_t preload_sig_batch_kernels() {
    return load_kernels(sig_persistent_kernel<64, 4, 1>, sig_persistent_kernel<64, 0, 1>,
                        sig_persistent_kernel<128, 4, 1>, sig_persistent_kernel<128, 0, 1>,
                        sig_persistent_kernel<128, 4, 3>, sig_persistent_kernel<128, 0, 3>,
                        sig_persistent_kernel<256, 4, 1>, sig_persistent_kernel<256, 0, 1>);
}

// Verify signatures four lanes each while the batch leaves the GPU idle
// (the same size rule as launch_ed25519_verify: up to 64 per SM).
cudaError_t launch_sig_batch(const SigWork& w_in, int threads, int blocks_per_sm, int sms, cudaStream_t s) {
    if (w_in.total_chunks == 0) return cudaSuccess;
    SigWork w = w_in;
    static const int forced = getenv("GB300_CRYPT_VERIFY_FORM") ? atoi(getenv("GB300_CRYPT_VERIFY_FORM")) : -1;
    const int form = (forced == kVerifySingle || forced == kVerifyQuad) ? forced : w.v_form_hint;
    // (with a device count, v.n is the capacity: the rule then uses the bound)
    w.v_quad = w.v.n > 0 &&
               (form == kVerifyQuad || (form != kVerifySingle && (uint64_t)w.v.n <= 64ull * (uint64_t)sms));
    cudaError_t e = cudaMemsetAsync(w.next, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    const bool half = w.v.window == 0;         // else window 4 (5 is not built for this kernel)
    // a launch with chunks for 3 blocks of 128 threads on every SM runs the
    // build capped at 3 blocks per SM (1 minimum otherwise).  Not a count_dev
    // launch: its size is a capacity, ~10x the signatures of a packet batch
    // (16,384 packets: 2.34 ms in the capped build against 1.66 ms).
    const uint64_t warps = (uint64_t)verify_chunks(w, w.v.n, w.v_quad) + sign_chunks(w);
    const bool full = threads != 64 && threads != 256 && blocks_per_sm < 1 && !w.count_dev &&
                      warps >= 12ull * (uint64_t)sms;
    // a count_dev launch sized above the four-lane limit still takes the
    // four-lane form when its device count turns out small
    w.v_quad_max = 0;
    if (w.count_dev && !w.v_quad && form != kVerifySingle) w.v_quad_max = (uint32_t)(64u * (uint32_t)sms);
    switch (threads) {
        case 64: return half ? launch_t<64, 0, 1>(w, blocks_per_sm, sms, s) : launch_t<64, 4, 1>(w, blocks_per_sm, sms, s);
        case 256:
            return half ? launch_t<256, 0, 1>(w, blocks_per_sm, sms, s) : launch_t<256, 4, 1>(w, blocks_per_sm, sms, s);
        default:
            if (full) return half ? launch_t<128, 0, 3>(w, blocks_per_sm, sms, s) : launch_t<128, 4, 3>(w, blocks_per_sm, sms, s);
            return half ? launch_t<128, 0, 1>(w, blocks_per_sm, sms, s) : launch_t<128, 4, 1>(w, blocks_per_sm, sms, s);
    }
}
