// noalloc.cu -- ALResidual (R = Fint(x) - lambda F) that allocates no device memory.
//
// Who needs it: callers that must not allocate device memory at the point where they need a
// residual -- a host framework that owns the whole device memory pool and forbids allocations
// outside it, or a service whose device footprint is fixed when it starts.  The regular
// klsa_al_residual grows its element-force buffer and staging vectors with cudaMalloc on first
// use; this variant takes caller-owned device vectors and keeps its only scratch -- the
// per-element internal forces -- in a fixed file-scope device array.
//
// Limits and sharing
//   * scratch: NOALLOC_SCRATCH_DOUBLES doubles (8 MiB) per GPU that loads the library, held
//     until the process exits; problems needing more (elements x 3(p+1)^2) are rejected.
//   * every call shares the array and it keeps the last call's contents; each call overwrites
//     every entry it reads, so nothing needs clearing.  Calls that overlap on the GPU (two host
//     threads, or two problems' streams) race on the array: serialise them.
//   * the call writes the problem's full-layout displacement vector (P.d_ufull), which the
//     problem's other entry points and solvers also write: no other call on the same problem
//     may overlap it.
//   * the kernels go to the problem's stream, which waits for no other stream: the caller
//     completes every pending write to d_x first.  The call synchronises that stream before it
//     returns.
//   * the first call on a device resolves the array's device address with
//     cudaGetSymbolAddress (once per device, with that device current).
#include <cuda_runtime.h>

#include <exception>
#include <mutex>
#include <string>

#include "../../include/klshell_gb300.h"
#include "problem.h"

namespace klsa {

constexpr size_t NOALLOC_SCRATCH_DOUBLES = size_t(1) << 20;
static __device__ __align__(256) double g_noalloc_elem_force[NOALLOC_SCRATCH_DOUBLES];

namespace {

constexpr int MAX_DEVICES = 64;
double* g_scratch_addr[MAX_DEVICES] = {};
std::mutex g_scratch_mutex;

// u_full[full(i)] = x_pub[i] for every free dof i (public order)
__global__ void noalloc_scatter_kernel(int nfree, const int* __restrict__ pub2int, const int* __restrict__ int2full,
                                       const double* __restrict__ x_pub, double* __restrict__ ufull) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nfree) ufull[int2full[pub2int[i]]] = x_pub[i];
}

// R_pub[i] = sum over the elements of dof i of the element force - lambda F
__global__ void noalloc_gather_kernel(int nfree, int p, int n1, int m1, int m2, int ncp, const int* __restrict__ pub2int,
                                      const int* __restrict__ int2full, const double* __restrict__ elemR,
                                      const double* __restrict__ F, double lambda, double* __restrict__ R_pub) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nfree) return;
    int id = pub2int[i];
    int fr = int2full[id];
    int ci = fr / ncp, A = fr - ci * ncp;
    int ia = A % n1, ja = A / n1;
    int NB1 = p + 1, D = 3 * NB1 * NB1;
    double s = 0.0;
    for (int e2 = max(ja - p, 0); e2 <= min(ja, m2 - 1); ++e2)
        for (int e1 = max(ia - p, 0); e1 <= min(ia, m1 - 1); ++e1) {
            int la = (ja - e2) * NB1 + (ia - e1);
            s += elemR[(size_t)(e2 * m1 + e1) * D + 3 * la + ci];
        }
    R_pub[i] = s - lambda * F[id];
}

}  // namespace

// Address of the scratch array on the current device (resolved once per device).
static int noalloc_scratch(double** out, std::string& err) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return KLSA_CUDA_ERROR; }
    if (dev < 0 || dev >= MAX_DEVICES) { err = "device index out of range"; return KLSA_UNSUPPORTED; }
    std::lock_guard<std::mutex> lk(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_elem_force);
        if (e != cudaSuccess) { err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e); return KLSA_CUDA_ERROR; }
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return KLSA_SUCCESS;
}

}  // namespace klsa

// defined in capi.cu
void klsa_set_error(const std::string& msg);
klsa::Problem* klsa_problem_impl(klsa_problem* prob);

extern "C" int klsa_al_residual_noalloc(klsa_problem* prob, const double* d_x, double lambda, double* d_R) {
    using namespace klsa;
    if (!prob || !d_x || !d_R) return KLSA_INVALID_ARGUMENT;
    Problem& P = *klsa_problem_impl(prob);
    const size_t need = (size_t)P.nel * 3 * (P.p + 1) * (P.p + 1);
    if (need > NOALLOC_SCRATCH_DOUBLES) {
        klsa_set_error("klsa_al_residual_noalloc: problem needs " + std::to_string(need) +
                       " doubles of element scratch, the no-allocation entry point holds at most " +
                       std::to_string(NOALLOC_SCRATCH_DOUBLES));
        return KLSA_INVALID_ARGUMENT;
    }
    std::string err;
    double* scratch = nullptr;
    int st = noalloc_scratch(&scratch, err);
    if (st != KLSA_SUCCESS) {
        klsa_set_error(err);
        return st;
    }
    try {
        const int threads = 256;
        noalloc_scatter_kernel<<<ceil_div(P.nfree, threads), threads, 0, P.stream>>>(P.nfree, P.d_pub2int.get(),
                                                                                 P.d_int2full.get(), d_x, P.d_ufull.get());
        count_launch();
        P.internal_force_elements(scratch);
        noalloc_gather_kernel<<<ceil_div(P.nfree, threads), threads, 0, P.stream>>>(
            P.nfree, P.p, P.n1, P.m1, P.m2, P.ncp, P.d_pub2int.get(), P.d_int2full.get(), scratch, P.d_F.get(), lambda,
            d_R);
        count_launch();
    } catch (const std::exception& ex) {
        klsa_set_error(ex.what());
        return KLSA_OTHER_ERROR;
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(P.stream);
    if (e != cudaSuccess) {
        klsa_set_error(cudaGetErrorString(e));
        return KLSA_CUDA_ERROR;
    }
    return KLSA_SUCCESS;
}
