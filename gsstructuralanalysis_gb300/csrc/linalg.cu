// linalg.cu -- FP64 vector kernels, multi-dot reductions and the named linear solvers.
#include "linalg.h"

#include <vector>

#include <algorithm>
#include <cmath>
#include <cstring>

namespace klsa {

namespace {

__global__ void to_f32_kernel(const double* __restrict__ x, float* __restrict__ y, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] = (float)x[i];
}
__global__ void to_f64_kernel(const float* __restrict__ x, double* __restrict__ y, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] = (double)x[i];
}
__global__ void axpby_kernel(double a, const double* __restrict__ x, double b, double* __restrict__ y, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] = a * x[i] + b * y[i];
}
__global__ void lincomb_kernel(double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                               double* __restrict__ z, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) z[i] = a * x[i] + b * y[i];
}

struct DotArgs {
    const double* x[8];
    const double* y[8];
};

constexpr int DOT_BLOCKS = 304;   // 2 x 152 SMs
constexpr int DOT_THREADS = 256;

// partial[b*npairs + k] = sum over the block's grid-stride slice of x_k . y_k (fixed order)
__global__ void __launch_bounds__(DOT_THREADS) multidot_kernel(DotArgs args, int npairs, int64_t n, double* partial) {
    __shared__ double red[8][DOT_THREADS / 32];
    double s[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) s[k] = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < npairs) s[k] += args.x[k][i] * args.y[k][i];
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        if (k < npairs) {
            double v = s[k];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) red[k][warp] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x < npairs) {
        double v = 0.0;
        for (int w = 0; w < DOT_THREADS / 32; ++w) v += red[threadIdx.x][w];
        partial[blockIdx.x * npairs + threadIdx.x] = v;
    }
}

// Jacobi (diagonal) preconditioner: z = r / diag
__global__ void diag_extract_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ cols,
                                    const float* __restrict__ vals, double* __restrict__ dinv) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double d = 0.0;
    for (int k = rowptr[r]; k < rowptr[r + 1]; ++k)
        if (cols[k] == r) d = vals[k];
    dinv[r] = d != 0.0 ? 1.0 / d : 1.0;
}
// Nodal block-Jacobi: the (up to 3 x 3) diagonal block of every control point's free dofs, which
// are consecutive in the internal order, inverted in FP64 (row-major, padded to 3 x 3).
__global__ void block_extract_kernel(int nblk, const int* __restrict__ start, const int* __restrict__ rowptr,
                                     const int* __restrict__ cols, const float* __restrict__ vals,
                                     double* __restrict__ binv) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    const int s0 = start[b], sz = start[b + 1] - s0;
    double A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, X[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < sz; ++i)
        for (int k = rowptr[s0 + i]; k < rowptr[s0 + i + 1]; ++k) {
            const int c = cols[k] - s0;
            if (c >= 0 && c < sz) A[i][c] = vals[k];
        }
    bool ok = true;
    for (int j = 0; j < sz; ++j) {            // Gauss-Jordan with partial pivoting
        int piv = j;
        for (int i = j + 1; i < sz; ++i)
            if (fabs(A[i][j]) > fabs(A[piv][j])) piv = i;
        if (A[piv][j] == 0.0) { ok = false; break; }
        for (int c = 0; c < 3; ++c) {
            double t = A[j][c]; A[j][c] = A[piv][c]; A[piv][c] = t;
            t = X[j][c]; X[j][c] = X[piv][c]; X[piv][c] = t;
        }
        const double inv = 1.0 / A[j][j];
        for (int c = 0; c < 3; ++c) { A[j][c] *= inv; X[j][c] *= inv; }
        for (int i = 0; i < sz; ++i) {
            if (i == j) continue;
            const double f = A[i][j];
            for (int c = 0; c < 3; ++c) { A[i][c] -= f * A[j][c]; X[i][c] -= f * X[j][c]; }
        }
    }
    for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c) binv[9 * (size_t)b + 3 * i + c] = ok ? X[i][c] : (i == c ? 1.0 : 0.0);
}
__global__ void block_apply_kernel(int nblk, const int* __restrict__ start, const double* __restrict__ binv,
                                   const double* __restrict__ r, double* __restrict__ z) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    const int s0 = start[b], sz = start[b + 1] - s0;
    const double* M = binv + 9 * (size_t)b;
    for (int i = 0; i < sz; ++i) {
        double v = 0.0;
        for (int c = 0; c < sz; ++c) v += M[3 * i + c] * r[s0 + c];
        z[s0 + i] = v;
    }
}
// z = a x + b y; z2 = z when z2 is given; acc += z when acc is given
__global__ void lincomb_ext_kernel(double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                                   double* __restrict__ z, double* __restrict__ z2, double* __restrict__ acc, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = a * x[i] + b * y[i];
    z[i] = v;
    if (z2) z2[i] = v;
    if (acc) acc[i] += v;
}
// the end of an accepted step: uprev = u; u += d; dold = d when dold is given
__global__ void step_finish_kernel(double* __restrict__ u, const double* __restrict__ d, double* __restrict__ uprev,
                                   double* __restrict__ dold, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double ui = u[i], di = d[i];
    uprev[i] = ui;
    u[i] = ui + di;
    if (dold) dold[i] = di;
}
__global__ void zero4_kernel(double* __restrict__ a, double* __restrict__ b, double* __restrict__ c,
                             double* __restrict__ d, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (a) a[i] = 0.0;
    if (b) b[i] = 0.0;
    if (c) c[i] = 0.0;
    if (d) d[i] = 0.0;
}
// the two right-hand sides [s0 b0, s1 b1] in FP32, and the two FP32 solutions back to FP64
__global__ void to_f32_pair_kernel(const double* __restrict__ b0, double s0, const double* __restrict__ b1, double s1,
                                   float* __restrict__ y, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    y[i] = (float)(s0 * b0[i]);
    y[n + i] = (float)(s1 * b1[i]);
}
__global__ void to_f64_pair_kernel(const float* __restrict__ x, double* __restrict__ x0, double* __restrict__ x1,
                                   int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    x0[i] = (double)x[i];
    x1[i] = (double)x[n + i];
}
__global__ void mul_kernel(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ c, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) c[i] = a[i] * b[i];
}

}  // namespace

namespace vec {

void to_f32(const double* x, float* y, int64_t n, cudaStream_t s) {
    to_f32_kernel<<<ceil_div(n, 256), 256, 0, s>>>(x, y, n);
    count_launch();
}
void to_f64(const float* x, double* y, int64_t n, cudaStream_t s) {
    to_f64_kernel<<<ceil_div(n, 256), 256, 0, s>>>(x, y, n);
    count_launch();
}
void axpby(double a, const double* x, double b, double* y, int64_t n, cudaStream_t s) {
    axpby_kernel<<<ceil_div(n, 256), 256, 0, s>>>(a, x, b, y, n);
    count_launch();
}
void lincomb(double a, const double* x, double b, const double* y, double* z, int64_t n, cudaStream_t s) {
    lincomb_kernel<<<ceil_div(n, 256), 256, 0, s>>>(a, x, b, y, z, n);
    count_launch();
}
void lincomb_ext(double a, const double* x, double b, const double* y, double* z, double* z2, double* acc, int64_t n,
                 cudaStream_t s) {
    lincomb_ext_kernel<<<ceil_div(n, 256), 256, 0, s>>>(a, x, b, y, z, z2, acc, n);
    count_launch();
}
void step_finish(double* u, const double* d, double* uprev, double* dold, int64_t n, cudaStream_t s) {
    step_finish_kernel<<<ceil_div(n, 256), 256, 0, s>>>(u, d, uprev, dold, n);
    count_launch();
}
void zero4(double* a, double* b, double* c, double* d, int64_t n, cudaStream_t s) {
    zero4_kernel<<<ceil_div(n, 256), 256, 0, s>>>(a, b, c, d, n);
    count_launch();
}

struct DotScratch {
    double* dev = nullptr;
    double* host = nullptr;
    DotScratch() {
        KL_CUDA(cudaMalloc(&dev, sizeof(double) * DOT_BLOCKS * 8));
        KL_CUDA(cudaMallocHost(&host, sizeof(double) * DOT_BLOCKS * 8));
    }
};

void multidot(int npairs, const double* const* xs, const double* const* ys, int64_t n, double* out, cudaStream_t s) {
    static thread_local DotScratch* scr = nullptr;
    if (!scr) scr = new DotScratch();
    DotArgs a;
    for (int k = 0; k < 8; ++k) {
        a.x[k] = k < npairs ? xs[k] : nullptr;
        a.y[k] = k < npairs ? ys[k] : nullptr;
    }
    multidot_kernel<<<DOT_BLOCKS, DOT_THREADS, 0, s>>>(a, npairs, n, scr->dev);
    count_launch();
    KL_CHECK_LAUNCH();
    KL_CUDA(cudaMemcpyAsync(scr->host, scr->dev, sizeof(double) * DOT_BLOCKS * npairs, cudaMemcpyDeviceToHost, s));
    KL_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < npairs; ++k) {
        double v = 0.0;
        for (int b = 0; b < DOT_BLOCKS; ++b) v += scr->host[b * npairs + k];
        out[k] = v;
    }
}

}  // namespace vec

// ------------------------------------------------------------------------------------------
// Multifrontal LDL^T (+ optional FP64 iterative refinement)
// ------------------------------------------------------------------------------------------
MFSolver::MFSolver(Problem& P, int refine, double refine_tol, bool fp64)
    : P_(P), refine_(refine), tol_(refine_tol), fp64_(fp64) {
    if (fp64_) P_.solver64();
    else P_.solver();
    int n = P_.nfree;
    b32_.alloc((size_t)n * MF_MAX_RHS);
    x32_.alloc((size_t)n * MF_MAX_RHS);
    r_.alloc((size_t)n * MF_MAX_RHS);
    dx_.alloc((size_t)n * MF_MAX_RHS);
}

int MFSolver::factor_current(bool f64_for_refine) {
    if (fp64_) {
        // FP64 fronts straight from the FP64 values
        if (P_.d_vals64.size() < (size_t)P_.nnz) throw std::logic_error("FP64 matrix values missing");
        has64_ = true;
        cudaEvent_t ev = g_timer.begin(P_.stream);
        P_.solver64().factorize_async(P_.d_vals64.get());
        g_timer.end(P_.stream, 1, ev);
        return P_.solver64().read_status();
    }
    // the caller assembled values into P_.d_vals32 (and d_vals64 when refining)
    if (f64_for_refine) {
        if (P_.d_vals64.size() < (size_t)P_.nnz) throw std::logic_error("FP64 matrix values missing");
        if (P_.d_vals32.size() < (size_t)P_.nnz) P_.d_vals32.alloc(P_.nnz);
        vec::to_f32(P_.d_vals64.get(), P_.d_vals32.get(), P_.nnz, P_.stream);
    } else if (P_.d_vals32.size() < (size_t)P_.nnz) {
        throw std::logic_error("FP32 matrix values missing");
    }
    has64_ = f64_for_refine;
    cudaEvent_t ev = g_timer.begin(P_.stream);
    P_.solver().factorize_async(P_.d_vals32.get());
    g_timer.end(P_.stream, 1, ev);
    return P_.solver().read_status();
}

uint64_t MFSolver::generation() const {
    if (fp64_) return P_.mf64 ? P_.mf64->generation() : 0;
    return P_.mf ? P_.mf->generation() : 0;
}

int MFSolver::compute_tangent() {
    cudaEvent_t ev = g_timer.begin(P_.stream);
    tangent_f64_ = refine_ > 0 || fp64_;
    if (tangent_f64_) P_.tangent_f64();
    else P_.tangent_f32();
    g_timer.end(P_.stream, 0, ev);
    return factor_current(refine_ > 0);
}

void MFSolver::solve_raw(const double* d_b, double* d_x, int nrhs) {
    int n = P_.nfree;
    cudaEvent_t ev = g_timer.begin(P_.stream);
    if (fp64_) {
        P_.solver64().solve(d_b, d_x, nrhs);
        g_timer.end(P_.stream, 2, ev);
        return;
    }
    vec::to_f32(d_b, b32_.get(), (int64_t)n * nrhs, P_.stream);
    P_.solver().solve(b32_.get(), x32_.get(), nrhs);
    vec::to_f64(x32_.get(), d_x, (int64_t)n * nrhs, P_.stream);
    g_timer.end(P_.stream, 2, ev);
}

int MFSolver::solve(const double* d_b, double* d_x, int nrhs) {
    if (nrhs < 1 || nrhs > MF_MAX_RHS) return ST_INVALID_ARGUMENT;
    solve_raw(d_b, d_x, nrhs);
    if (refine_ <= 0 || !has64_) return ST_SUCCESS;
    int n = P_.nfree;
    std::vector<double> bn(nrhs);
    {
        const double* xs[MF_MAX_RHS];
        for (int q = 0; q < nrhs; ++q) xs[q] = d_b + (size_t)q * n;
        vec::multidot(nrhs, xs, xs, n, bn.data(), P_.stream);
    }
    last_refine_its_ = 0;
    for (int it = 0; it < refine_; ++it) {
        for (int q = 0; q < nrhs; ++q) {
            spmv(P_, true, d_x + (size_t)q * n, r_.get() + (size_t)q * n);
            vec::axpby(1.0, d_b + (size_t)q * n, -1.0, r_.get() + (size_t)q * n, n, P_.stream);
        }
        std::vector<double> rn(nrhs);
        const double* rs[MF_MAX_RHS];
        for (int q = 0; q < nrhs; ++q) rs[q] = r_.get() + (size_t)q * n;
        vec::multidot(nrhs, rs, rs, n, rn.data(), P_.stream);
        bool done = true;
        for (int q = 0; q < nrhs; ++q)
            if (std::sqrt(rn[q]) > tol_ * std::sqrt(bn[q])) done = false;
        if (done) break;
        solve_raw(r_.get(), dx_.get(), nrhs);
        vec::axpby(1.0, dx_.get(), 1.0, d_x, (int64_t)n * nrhs, P_.stream);
        ++last_refine_its_;
    }
    return ST_SUCCESS;
}

bool MFSolver::solve_pair(const double* b0, double s0, const double* b1, double s1, double* x0, double* x1) {
    // only the plain FP32-front solve: refinement and FP64 fronts take the generic path
    if (fp64_ || (refine_ > 0 && has64_)) return false;
    const int64_t n = P_.nfree;
    cudaEvent_t ev = g_timer.begin(P_.stream);
    to_f32_pair_kernel<<<ceil_div(n, 256), 256, 0, P_.stream>>>(b0, s0, b1, s1, b32_.get(), n);
    count_launch();
    P_.solver().solve(b32_.get(), x32_.get(), 2);
    to_f64_pair_kernel<<<ceil_div(n, 256), 256, 0, P_.stream>>>(x32_.get(), x0, x1, n);
    count_launch();
    KL_CHECK_LAUNCH();
    g_timer.end(P_.stream, 2, ev);
    last_refine_its_ = 0;
    return true;
}

void MFSolver::stability(double* min_d, int64_t* neg) {
    if (fp64_) P_.solver64().stability(min_d, neg);
    else P_.solver().stability(min_d, neg);
}

// ------------------------------------------------------------------------------------------
// Jacobi-preconditioned CG ("CGDiagonal": Eigen ConjugateGradient + DiagonalPreconditioner)
// ------------------------------------------------------------------------------------------
PCGSolver::PCGSolver(Problem& P, int max_it, double tol, bool block)
    : P_(P), max_it_(max_it), tol_(tol), block_(block) {
    int n = P_.nfree;
    dinv_.alloc(n); r_.alloc(n); z_.alloc(n); p_.alloc(n); q_.alloc(n);
    if (max_it_ <= 0) max_it_ = 2 * n;
    if (block_) {
        // blocks: runs of consecutive internal dofs of one control point
        std::vector<int> i2f(n);
        P_.d_int2full.download(i2f.data(), n, P_.stream);
        KL_CUDA(cudaStreamSynchronize(P_.stream));
        std::vector<int> start;
        for (int i = 0; i < n; ++i)
            if (i == 0 || i2f[i] % P_.ncp != i2f[i - 1] % P_.ncp || i - start.back() == 3) start.push_back(i);
        start.push_back(n);
        nblk_ = (int)start.size() - 1;
        blk_start_.upload(start, P_.stream);
        binv_.alloc((size_t)9 * nblk_);
    }
}

void PCGSolver::precondition(const double* r, double* z) {
    if (block_) {
        block_apply_kernel<<<ceil_div(nblk_, 256), 256, 0, P_.stream>>>(nblk_, blk_start_.get(), binv_.get(), r, z);
    } else {
        mul_kernel<<<ceil_div(P_.nfree, 256), 256, 0, P_.stream>>>(dinv_.get(), r, z, P_.nfree);
    }
    count_launch();
}

int PCGSolver::compute_tangent() {
    P_.tangent_f32();
    if (block_) {
        block_extract_kernel<<<ceil_div(nblk_, 256), 256, 0, P_.stream>>>(nblk_, blk_start_.get(), P_.d_rowptr.get(),
                                                                         P_.d_cols.get(), P_.d_vals32.get(), binv_.get());
    } else {
        diag_extract_kernel<<<ceil_div(P_.nfree, 256), 256, 0, P_.stream>>>(P_.nfree, P_.d_rowptr.get(), P_.d_cols.get(),
                                                                             P_.d_vals32.get(), dinv_.get());
    }
    count_launch();
    return ST_SUCCESS;
}

int PCGSolver::solve(const double* d_b, double* d_x, int nrhs) {
    int n = P_.nfree;
    cudaStream_t s = P_.stream;
    for (int q = 0; q < nrhs; ++q) {
        const double* b = d_b + (size_t)q * n;
        double* x = d_x + (size_t)q * n;
        KL_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
        KL_CUDA(cudaMemcpyAsync(r_.get(), b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        precondition(r_.get(), z_.get());
        KL_CUDA(cudaMemcpyAsync(p_.get(), z_.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        double d[2];
        const double* xs[2] = {r_.get(), b};
        const double* ys[2] = {z_.get(), b};
        vec::multidot(2, xs, ys, n, d, s);
        double rz = d[0], bb = d[1];
        if (bb == 0.0) continue;
        iterations_ = 0;
        for (int it = 0; it < max_it_; ++it) {
            spmv(P_, false, p_.get(), q_.get());
            double pq;
            const double* a1[1] = {p_.get()};
            const double* a2[1] = {q_.get()};
            vec::multidot(1, a1, a2, n, &pq, s);
            double alpha = rz / pq;
            vec::axpby(alpha, p_.get(), 1.0, x, n, s);
            vec::axpby(-alpha, q_.get(), 1.0, r_.get(), n, s);
            precondition(r_.get(), z_.get());
            double dd[2];
            const double* u1[2] = {r_.get(), r_.get()};
            const double* u2[2] = {z_.get(), r_.get()};
            vec::multidot(2, u1, u2, n, dd, s);
            iterations_ = it + 1;
            if (std::sqrt(dd[1]) <= tol_ * std::sqrt(bb)) break;
            double beta = dd[0] / rz;
            rz = dd[0];
            vec::axpby(1.0, z_.get(), beta, p_.get(), n, s);
        }
    }
    return ST_SUCCESS;
}

std::unique_ptr<LinearSolver> make_linear_solver(Problem& P, const std::string& name, int refine, double refine_tol,
                                                 int cg_max_it, double cg_tol, int front_precision) {
    if (front_precision != 32 && front_precision != 64) throw std::invalid_argument("FrontPrecision must be 32 or 64");
    if (name == "SimplicialLDLT" || name == "GPUMultifrontalLDLT" || name == "SimplicialLLT" || name == "LDLT")
        return std::unique_ptr<LinearSolver>(new MFSolver(P, refine, refine_tol, front_precision == 64));
    if (name == "CGDiagonal" || name == "ConjugateGradient")
        return std::unique_ptr<LinearSolver>(new PCGSolver(P, cg_max_it, cg_tol, false));
    if (name == "GPUPCG" || name == "BlockJacobiCG")
        return std::unique_ptr<LinearSolver>(new PCGSolver(P, cg_max_it, cg_tol, true));
    return nullptr;
}

}  // namespace klsa
