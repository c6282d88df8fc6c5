// Grow-only device and page-locked host buffers (host side of the library).
//
// Growing never synchronises the device: device memory is replaced with the
// stream-ordered allocator (cudaFreeAsync / cudaMallocAsync on the stream
// that uses the buffer), and a replaced page-locked buffer is kept until
// release() instead of being freed while copies from it may be in flight.
// (cudaFree / cudaFreeHost wait for all work on the device, which would
// stall every stream behind, say, a second-long PoH chain.)
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include <vector>

namespace gb300 {

inline size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

inline size_t grow_size(size_t bytes) { return round_up(bytes < 4096 ? 4096 : bytes + bytes / 4, 4096); }

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes, cudaStream_t s = 0) {
        if (p && bytes <= cap) return cudaSuccess;
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
        cap = 0;
        const size_t want = grow_size(bytes);
        cudaError_t e = cudaMallocAsync(&p, want, s);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        cap = want;
        return cudaSuccess;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct HostBuf {
    void* p = nullptr;
    size_t cap = 0;
    std::vector<void*> retired;
    cudaError_t ensure(size_t bytes) {
        if (p && bytes <= cap) return cudaSuccess;
        if (p) retired.push_back(p);
        p = nullptr;
        cap = 0;
        const size_t want = grow_size(bytes);
        cudaError_t e = cudaMallocHost(&p, want);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        cap = want;
        return cudaSuccess;
    }
    void release() {
        if (p) cudaFreeHost(p);
        for (void* r : retired) cudaFreeHost(r);
        retired.clear();
        p = nullptr;
        cap = 0;
    }
};

}  // namespace gb300
