// Growable device buffer: reserve() reallocates only when the requested
// number of elements exceeds the capacity, so steady-state calls allocate
// nothing.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cuda_runtime.h>

namespace iss {

template <typename T>
struct DevBuf {
    T* ptr = nullptr;
    size_t cap = 0;   // elements
    cudaError_t reserve(size_t n) {
        if (n <= cap && ptr) return cudaSuccess;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(n, 1);
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&ptr), want * sizeof(T));
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
    }
};

}  // namespace iss
