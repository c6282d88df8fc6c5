// Grow-only device and page-locked host buffers (host side of the library).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace gb300 {

inline size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (p && bytes <= cap) return cudaSuccess;
        release();
        size_t want = round_up(bytes < 4096 ? 4096 : bytes + bytes / 4, 4096);
        cudaError_t e = cudaMalloc(&p, want);
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
    cudaError_t ensure(size_t bytes) {
        if (p && bytes <= cap) return cudaSuccess;
        release();
        size_t want = round_up(bytes < 4096 ? 4096 : bytes + bytes / 4, 4096);
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
        p = nullptr;
        cap = 0;
    }
};


}  // namespace gb300
