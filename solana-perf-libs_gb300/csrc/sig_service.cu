// Resident signature service kernel of the served loop (server.cu).
//
// The reference serves one synchronous batch per call: a launch sized to the
// batch, then a copy back and a stream synchronisation
// (src/cuda-ecc-ed25519/verify.cu:289-334, over the context pool of
// gpu_ctx.cu:46-73).  A served loop that merges arriving requests into such
// launches makes every request wait for its whole merged launch, and a launch
// that fills the GPU waits for the previous one's blocks to drain.  Here one
// long-lived launch keeps warps resident; they take 32-item chunks from a
// FIFO in publication order, so the oldest work runs first, and each request
// is complete (results in host memory, completion word written) as soon as
// its own last chunk is, whatever else is in flight.
//
// Protocol (host side in server.cu):
//   * the host fills a request slot and its chunk descriptors in page-locked
//     memory, copies the packets and per-signature arrays into device memory
//     on one stream, then advances SvcDevice::tail with a stream write
//     ordered after those copies (the write is preceded by a system-wide
//     fence, so a warp that reads the new tail with acquire semantics sees
//     the inputs and the descriptors);
//   * a warp claims the next chunk by compare-and-swap on `head`, runs it,
//     fences its result stores, and adds its item count to the request's
//     counter; the warp that completes the count resets it for the slot's
//     next request, fences, and writes the request's generation number into
//     its completion word in host memory;
//   * every wait is bounded, and the launch leaves as a whole: once no warp
//     has claimed a chunk for idle_ns and the FIFO is empty (or `stop` is
//     set), the first warp to notice sets `exiting` and every warp leaves at
//     its next look; the host resets the flag and launches the kernel again
//     when work arrives and no launch is running.  (Warps that left one by
//     one after their own idle time would leave a launch of a few warps
//     running, which the host cannot see, to carry a later burst alone.)
#include <cuda_runtime.h>
#include <atomic>
#include <cstring>
#include "kernels.h"
#include "tables.cuh"
#include "sha512.cuh"
#include "sc25519.cuh"

namespace {

#include "ed25519_ops.cuh"
#include "verify_quad.cuh"

constexpr size_t kSvcCombBytes = sizeof(ge_niels) * COMB_WINDOWS * COMB_ENTRIES;
constexpr int kSvcThreads = 128;

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t ld_acquire_sys(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint32_t ld_relaxed_gpu(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint64_t ld_relaxed_gpu64(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_sys(uint32_t* p, uint32_t v) {
    asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Descriptors and request slots are rewritten by the host while the kernel
// runs (after their previous use has completed), so they are read with
// volatile loads: never from a cache line an earlier read left behind, and
// never through the read-only data path.
__device__ __forceinline__ uint4 ld_volatile_v4(const void* p) {
    uint4 v;
    asm volatile("ld.volatile.global.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p)
                 : "memory");
    return v;
}

template <class S>
__device__ __forceinline__ S ld_volatile_struct(const S* p) {
    static_assert(sizeof(S) % 16 == 0 && alignof(S) <= 16, "read as 16-byte words");
    uint4 w[sizeof(S) / 16];
#pragma unroll
    for (int k = 0; k < (int)(sizeof(S) / 16); k++) w[k] = ld_volatile_v4(reinterpret_cast<const uint4*>(p) + k);
    S s;
    memcpy(&s, w, sizeof(S));
    return s;
}

// The next published chunk, claimed for the warp; false once the launch is
// leaving.  Polls device memory only, backing off from 256 ns to 4 us
// between looks.  Called by the whole warp: lane 0 makes each attempt as
// straight-line code, the outcome is broadcast, and the loop (sleeps
// included) runs on every lane, so the warp leaves it converged.  With the
// polling loop inside a lane-0-only branch, lanes 1-31 went ahead without
// lane 0 and the warp stayed split in two for the whole chunk: measured on
// GB300 with ncu, the four-lane verify then issued twice its instructions
// with ~20 active threads and 2.6 branch-resolution stalls per issue, and
// eight signatures took 3.0 ms against 0.46 ms in a plain launch.
__device__ __forceinline__ bool claim_chunk(const SvcParams& p, uint32_t lane, uint32_t& c, uint64_t t_start,
                                            bool first, uint32_t slot, bool& preferred) {
    uint32_t sleep_ns = 256;
    for (;;) {
        uint32_t r = 3, got = 0;      // 0 leave, 1 claimed (4: by a preferred warp), 2 lost a race, 3 empty
        if (lane == 0) {
            if (ld_relaxed_gpu(&p.dev->exiting)) {
                r = 0;
            } else {
                const uint32_t t = ld_relaxed_gpu(&p.dev->tail);
                const uint32_t h = ld_relaxed_gpu(&p.dev->head);
                // preferred: a first-block warp on a sub-partition without
                // a PoH round warp.  Any other warp takes a chunk only when
                // the waiting chunks outnumber the idle preferred warps.
                const int32_t waiting = (int32_t)(t - h);
                const bool pref = first && ld_relaxed_gpu(p.poh_slots + slot) == 0u;
                const int32_t n_pref = (int32_t)p.first_warps - (int32_t)ld_relaxed_gpu(p.poh_busy_slots);
                const bool mine = waiting > 0 &&
                                  (pref || waiting > n_pref - (int32_t)ld_relaxed_gpu(&p.dev->busy_first));
                if (mine) {
                    if (atomicCAS(&p.dev->head, h, h + 1u) == h) {
                        r = pref ? 4u : 1u;
                        got = h;
                        atomicMax(reinterpret_cast<unsigned long long*>(&p.dev->last_claim_ns),
                                  (unsigned long long)global_ns());
                    } else {
                        r = 2;
                    }
                } else if (waiting <= 0) {
                    const uint64_t last = ld_relaxed_gpu64(&p.dev->last_claim_ns);
                    const uint64_t since = last > t_start ? last : t_start;
                    const uint64_t now = global_ns();
                    if (ld_relaxed_gpu(&p.dev->stop) || (now > since && now - since > p.idle_ns)) {
                        atomicExch(&p.dev->exiting, 1u);
                        r = 0;
                    }
                }
            }
        }
        r = __shfl_sync(0xffffffffu, r, 0);
        if (r == 0) return false;
        if (r == 1 || r == 4) {
            c = __shfl_sync(0xffffffffu, got, 0);
            preferred = r == 4;
            return true;
        }
        if (r == 3) {
            __nanosleep(sleep_ns);
            if (sleep_ns < 4096) sleep_ns <<= 1;
        }
    }
}

// At most 216 registers a thread (__maxnreg__, which excludes
// __launch_bounds__; launched with 128 threads): the four-lane verify keeps
// its registers without spilling, and two blocks per SM (55,296 registers)
// leave room for the PoH pair blocks that run beside them.  A 168-register
// build (three blocks per SM) spilled in the four-lane path.
template <int T, int W>
__global__ void __maxnreg__(216) sig_service_kernel(SvcParams p) {
    __shared__ uint32_t sVB[VB_WORDS * VB_ENTRIES];
    __shared__ uint32_t s_rank;
    extern __shared__ uint4 s_comb4[];
    if (threadIdx.x == 0) {
        // this block's rank among the launch's blocks on its SM
        uint32_t smid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        s_rank = atomicAdd(&p.dev->sm_blocks[smid & 255u], 1u);
    }
    for (int k = threadIdx.x; k < VB_WORDS * VB_ENTRIES; k += blockDim.x) sVB[k] = p.tables->vb[k];
    {
        const uint4* g = reinterpret_cast<const uint4*>(&p.tables->comb[0][0]);
        for (uint32_t k = threadIdx.x; k < kSvcCombBytes / 16; k += blockDim.x) s_comb4[k] = g[k];
    }
    __syncthreads();
    const ge_niels* comb = reinterpret_cast<const ge_niels*>(s_comb4);
    const uint32_t lane = threadIdx.x & 31u;
    // The first block on each SM has one warp on each sub-partition; its
    // warps take chunks first, so that a few chunks spread over the SMs'
    // sub-partitions instead of doubling up on some while others idle (a
    // verify chain is latency-bound: a second warp on the same
    // sub-partition slows both), and among them those whose sub-partition
    // runs no PoH round warp.
    const bool first = s_rank == 0;
    uint32_t slot;
    {
        uint32_t smid, wid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        asm volatile("mov.u32 %0, %%warpid;" : "=r"(wid));
        slot = ((smid % kMaxServeSms) << 2) | (wid & 3u);  // as the PoH kernels count it
    }
    const uint64_t t_start = global_ns();
    if (lane == 0) atomicAdd(&p.dev->warps, 1u);
    for (;;) {
        uint32_t c = 0;
        bool preferred = false;
        if (!claim_chunk(p, lane, c, t_start, first, slot, preferred)) break;
        if (preferred && lane == 0) atomicAdd(&p.dev->busy_first, 1u);
        // every lane synchronises with the publication of chunk c (the
        // stream write of tail after the input copies): its later loads of
        // the descriptors (host memory) and inputs (device memory) see them
        (void)ld_acquire_sys(&p.dev->tail);
        const SvcChunk ch = ld_volatile_struct(p.ring + (c & (p.ring_size - 1u)));
        if (lane == 0)
            atomicMin(reinterpret_cast<unsigned long long*>(p.first_claim + ch.req), (unsigned long long)global_ns());
        const SvcReq rq = ld_volatile_struct(p.req + ch.req);
        const SigBatch& b = rq.b;
        const uint32_t gen = rq.gen;
        if (ch.mode == kSvcVerifyQuad) {
            // every lane runs an item (past the end: the chunk's last again,
            // result dropped) so the whole warp meets every shuffle
            const uint32_t q = lane >> 2;
            const uint32_t i = ch.first + (q < ch.count ? q : ch.count - 1u);
            const bool ok = verify_quad(b, sVB, i, lane & 3u);
            if (q < ch.count && (lane & 3u) == 0) b.out[i] = ok ? 1 : 0;
        } else if (ch.mode == kSvcSign) {
            if (lane < ch.count) sign_one_tab(b, ch.first + lane, comb);
        } else {
            // every lane runs an item (past the end: the chunk's last
            // again, result dropped): the half-size-scalar form votes over
            // the warp
            const uint32_t i = ch.first + (lane < ch.count ? lane : ch.count - 1u);
            const bool ok = verify_window<W>(b, sVB, i);
            if (lane < ch.count) b.out[i] = ok ? 1 : 0;
        }
        if (preferred && lane == 0) atomicSub(&p.dev->busy_first, 1u);
        // results (host memory) before the count; the completing warp
        // resets the slot's counter, then publishes the completion word
        __threadfence_system();
        __syncwarp();
        if (lane == 0) {
            const uint32_t before = atomicAdd(&p.items_done[ch.req], ch.count);
            if (before + ch.count == b.n) {
                atomicExch(&p.items_done[ch.req], 0u);
                const uint64_t t_first =
                    atomicExch(reinterpret_cast<unsigned long long*>(p.first_claim + ch.req), ~0ull);
                p.times[2 * ch.req] = t_first;
                p.times[2 * ch.req + 1] = global_ns();
                __threadfence_system();
                st_release_sys(&p.done[ch.req], gen);
            }
        }
    }
}

// one-lane chunks with half-size scalars (verify_half.cuh)
#define SVC_KERNEL sig_service_kernel<kSvcThreads, 0>

// %globaltimer now, for relating the kernel's times to the host clock.
__global__ void svc_clock_kernel(uint64_t* out) { *reinterpret_cast<volatile uint64_t*>(out) = global_ns(); }

}  // namespace

cudaError_t preload_sig_service_kernels() { return load_kernels(SVC_KERNEL, svc_clock_kernel); }

cudaError_t launch_svc_clock(uint64_t* out, cudaStream_t s) {
    svc_clock_kernel<<<1, 1, 0, s>>>(out);
    return cudaGetLastError();
}

cudaError_t sig_service_blocks_per_sm(int* blocks) {
    static std::atomic<uint64_t> opted{0};      // bit d: the attributes are set on device d
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = 1ull << (dev & 63);
    if (!(opted.load() & bit)) {
        e = cudaFuncSetAttribute(SVC_KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSvcCombBytes);
        if (e != cudaSuccess) return e;
        // the same L1 / shared split as the PoH kernels it runs beside
        // (poh_batch.cu), so neither waits for the other to drain an SM
        // (kernels.h gives the sizes)
        e = cudaFuncSetAttribute(SVC_KERNEL, cudaFuncAttributePreferredSharedMemoryCarveout, kServeCarveoutPercent);
        if (e != cudaSuccess) return e;
        opted.fetch_or(bit);
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, SVC_KERNEL, kSvcThreads, kSvcCombBytes);
}

cudaError_t launch_sig_service(const SvcParams& p, int blocks_per_sm, int sms, cudaStream_t s) {
    int maxb = 0;
    cudaError_t e = sig_service_blocks_per_sm(&maxb);
    if (e != cudaSuccess) return e;
    if (maxb < 1) return cudaErrorInvalidConfiguration;
    const int b = blocks_per_sm < 1 ? maxb : (blocks_per_sm < maxb ? blocks_per_sm : maxb);
    SVC_KERNEL<<<(unsigned)(b * sms), kSvcThreads, kSvcCombBytes, s>>>(p);
    return cudaGetLastError();
}
