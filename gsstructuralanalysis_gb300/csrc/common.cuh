// common.cuh -- shared helpers for the sm_103a Kirchhoff-Love shell library.
#pragma once

#include <atomic>
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

// RAII page-locked host buffer
template <class T>
struct PinnedBuf {
    T* ptr = nullptr;
    explicit PinnedBuf(size_t count = 1) { KL_CUDA(cudaMallocHost(&ptr, count * sizeof(T))); }
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() { if (ptr) cudaFreeHost(ptr); }
    T* get() const { return ptr; }
};

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

// Launch counter for the kernels of this library (reported by the benchmark).  Several host
// threads may drive separate problems at once, so the counter is atomic; while a thread captures
// a graph, its launches go to that capture's own counter (CaptureCount) instead.
extern std::atomic<unsigned long long> g_launch_count;
extern thread_local unsigned long long* t_capture_count;
inline void count_launch(unsigned long long k = 1) {
    if (t_capture_count)
        *t_capture_count += k;
    else
        g_launch_count.fetch_add(k, std::memory_order_relaxed);
}
struct CaptureCount {
    unsigned long long n = 0;
    unsigned long long* prev;
    CaptureCount() : prev(t_capture_count) { t_capture_count = &n; }
    ~CaptureCount() { t_capture_count = prev; }
    CaptureCount(const CaptureCount&) = delete;
    CaptureCount& operator=(const CaptureCount&) = delete;
};

}  // namespace klsa

namespace klsa {

// Optional per-phase device timing with CUDA events on the launching stream.
// Phases: 0 tangent assembly, 1 factorisation, 2 triangular solves, 3 residual (Fint),
//         4 multifrontal trailing-update launches, 5 multifrontal diagonal launches,
//         6 multifrontal panel launches, 7 eigen / other.
struct PhaseTimer {
    static constexpr int NPH = 8;
    bool enabled = false;
    double ms[NPH] = {0};
    unsigned long long count[NPH] = {0};
    std::vector<cudaEvent_t> pool;
    struct Pending { int ph; cudaEvent_t a, b; };
    std::vector<Pending> pending;
    cudaEvent_t get() {
        if (pool.empty()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            return e;
        }
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t begin(cudaStream_t s) {
        if (!enabled) return nullptr;
        cudaEvent_t a = get();
        cudaEventRecord(a, s);
        return a;
    }
    void end(cudaStream_t s, int ph, cudaEvent_t a) {
        if (!enabled || !a) return;
        cudaEvent_t b = get();
        cudaEventRecord(b, s);
        pending.push_back({ph, a, b});
        if (pending.size() > 4096) collect();
    }
    void collect() {
        for (auto& p : pending) {
            float t = 0;
            cudaEventSynchronize(p.b);
            cudaEventElapsedTime(&t, p.a, p.b);
            ms[p.ph] += t;
            count[p.ph] += 1;
            pool.push_back(p.a);
            pool.push_back(p.b);
        }
        pending.clear();
    }
    void reset() {
        collect();
        for (int i = 0; i < NPH; ++i) { ms[i] = 0; count[i] = 0; }
    }
};
extern PhaseTimer g_timer;

}  // namespace klsa
