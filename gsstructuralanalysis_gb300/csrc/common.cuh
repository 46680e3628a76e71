// common.cuh -- shared helpers for the sm_103a Kirchhoff-Love shell library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

namespace klsa {

// Status codes of the C-ABI.  0..5 mirror gsStatus
// (gsStructuralAnalysisTools/gsStructuralAnalysisTypes.h:22-30); negative codes are ABI errors.
enum Status : int {
    ST_SUCCESS = 0,
    ST_NOT_CONVERGED = 1,
    ST_ASSEMBLY_ERROR = 2,
    ST_SOLVER_ERROR = 3,
    ST_NOT_STARTED = 4,
    ST_OTHER_ERROR = 5,
    ST_INVALID_ARGUMENT = -1,
    ST_CUDA_ERROR = -2,
    ST_UNSUPPORTED = -3,
};

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

#define KL_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t _e = (call);                                                               \
        if (_e != cudaSuccess)                                                                 \
            throw ::klsa::CudaError(std::string(#call) + ": " + cudaGetErrorString(_e));       \
    } while (0)

#define KL_CHECK_LAUNCH() KL_CUDA(cudaGetLastError())

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// RAII device buffer
template <class T>
struct DevBuf {
    T* ptr = nullptr;
    size_t n = 0;
    DevBuf() = default;
    explicit DevBuf(size_t count) { alloc(count); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : ptr(o.ptr), n(o.n) { o.ptr = nullptr; o.n = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) { release(); ptr = o.ptr; n = o.n; o.ptr = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t count) {
        release();
        n = count;
        if (count) KL_CUDA(cudaMalloc(&ptr, count * sizeof(T)));
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        n = 0;
    }
    void upload(const T* h, size_t count, cudaStream_t s = 0) {
        if (count > n) alloc(count);
        if (count) KL_CUDA(cudaMemcpyAsync(ptr, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void upload(const std::vector<T>& v, cudaStream_t s = 0) { upload(v.data(), v.size(), s); }
    void download(T* h, size_t count, cudaStream_t s = 0) const {
        if (count) KL_CUDA(cudaMemcpyAsync(h, ptr, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    void zero(cudaStream_t s = 0) {
        if (n) KL_CUDA(cudaMemsetAsync(ptr, 0, n * sizeof(T), s));
    }
    T* get() const { return ptr; }
    size_t size() const { return n; }
};

// Launch counter for the kernels of this library (reported by the benchmark).
extern unsigned long long g_launch_count;
inline void count_launch(unsigned long long k = 1) { g_launch_count += k; }

}  // namespace klsa
