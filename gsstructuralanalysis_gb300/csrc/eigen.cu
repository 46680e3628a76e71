// eigen.cu -- thick-restart Lanczos with FP64 full reorthogonalisation for the generalised
// symmetric pencil A v = lambda B v, in the five operator modes of gsEigenProblemBase::computeSparse
// (gsEigenProblemBase.hpp:54-215, the Spectra GEigsMode variants; Spectra itself is not in the
// reference tree, so its documented operators are restated):
//   0 Cholesky, 1 RegularInverse (B SPD): op = B^-1 (A - sigma B), nu = lambda - sigma
//   2 ShiftInvert (B SPD):                 op = (A - sigma B)^-1 B, nu = 1/(lambda - sigma)
//   3 Buckling (A SPD):                    op = (A - sigma B)^-1 A, nu = lambda/(lambda - sigma)
//   4 Cayley (B SPD):                      op = (A - sigma B)^-1 (A + sigma B) = I + 2 sigma (A - sigma B)^-1 B,
//                                          nu = (lambda + sigma)/(lambda - sigma)
// The Lanczos basis is orthonormal in the C-inner product (C = A for Buckling, B otherwise); Cayley
// runs the shift-invert recurrence (the same Krylov space) and selects by its own nu.  The
// selection rule (Spectra SortRule: 0 LargestMagn, 1 LargestReal, 3 LargestAlge, 4 SmallestMagn,
// 5 SmallestReal, 7 SmallestAlge, 8 BothEnds) picks the wanted operator eigenvalues nu; the sort
// rule orders the back-transformed lambda.  The factorised matrix is factorised once by the
// multifrontal LDL^T (FP64 fronts by default, FP32 + FP64 refinement on request).  V and Y = C V
// stay in HBM (FP64); reorthogonalisation is classical Gram-Schmidt done twice with batched dot
// products; the small projected matrix is diagonalised on the host by cyclic Jacobi in FP64.
#include "eigen.h"

#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace klsa {

namespace {

__global__ void spmv_vals_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ cols,
                                 const double* __restrict__ vals, const double* __restrict__ x, double* __restrict__ y) {
    int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (row >= n) return;
    double s = 0.0;
    for (int k = rowptr[row] + lane; k < rowptr[row + 1]; k += 32) s += vals[k] * x[cols[k]];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) y[row] = s;
}

constexpr int GB = 304;   // blocks of the batched dot kernel

// partial[b*m + i] = sum_{rows of block b} Y[:, i] . w
__global__ void batched_dot_kernel(int n, int m, const double* __restrict__ Y, const double* __restrict__ w,
                                   double* __restrict__ partial) {
    extern __shared__ double sred[];   // m * (blockDim/32)
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = 0; i < m; ++i) {
        double s = 0.0;
        for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
            s += Y[(size_t)i * n + r] * w[r];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) sred[i * nw + warp] = s;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < nw; ++k) s += sred[i * nw + k];
        partial[(size_t)blockIdx.x * m + i] = s;
    }
}

// w -= V h   (V: n x m column-major)
__global__ void gemv_sub_kernel(int n, int m, const double* __restrict__ V, const double* __restrict__ h, double* w) {
    extern __shared__ double hs[];
    for (int i = threadIdx.x; i < m; i += blockDim.x) hs[i] = h[i];
    __syncthreads();
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double s = 0.0;
    for (int i = 0; i < m; ++i) s += V[(size_t)i * n + r] * hs[i];
    w[r] -= s;
}

// out[:, j] = V S[:, j], j < k (S: m x k column-major)
__global__ void gemm_vs_kernel(int n, int m, int k, const double* __restrict__ V, const double* __restrict__ S,
                               double* __restrict__ out) {
    extern __shared__ double Ss[];
    for (int i = threadIdx.x; i < m * k; i += blockDim.x) Ss[i] = S[i];
    __syncthreads();
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (int j = 0; j < k; ++j) {
        double s = 0.0;
        for (int i = 0; i < m; ++i) s += V[(size_t)i * n + r] * Ss[j * m + i];
        out[(size_t)j * n + r] = s;
    }
}

__global__ void combine_kernel(int64_t n, double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                               double* __restrict__ z) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) z[i] = a * x[i] + b * y[i];
}

// values of the identity matrix on the CSR pattern (the pattern always holds the diagonal)
__global__ void identity_vals_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ cols,
                                     double* __restrict__ vals) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) vals[k] = (cols[k] == r) ? 1.0 : 0.0;
}

// cyclic Jacobi eigen-decomposition of a symmetric m x m matrix (row-major H, column eigvecs in Q)
void jacobi_eig(int m, std::vector<double> H, std::vector<double>& w, std::vector<double>& Q) {
    Q.assign((size_t)m * m, 0.0);
    for (int i = 0; i < m; ++i) Q[(size_t)i * m + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < m; ++j) {
                double v = H[(size_t)i * m + j] * H[(size_t)i * m + j];
                tot += v;
                if (i != j) off += v;
            }
        if (off <= 1e-30 * tot || off == 0.0) break;
        for (int p = 0; p < m - 1; ++p)
            for (int q = p + 1; q < m; ++q) {
                double apq = H[(size_t)p * m + q];
                if (std::fabs(apq) < 1e-300) continue;
                double app = H[(size_t)p * m + p], aqq = H[(size_t)q * m + q];
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < m; ++k) {
                    double hkp = H[(size_t)k * m + p], hkq = H[(size_t)k * m + q];
                    H[(size_t)k * m + p] = c * hkp - s * hkq;
                    H[(size_t)k * m + q] = s * hkp + c * hkq;
                }
                for (int k = 0; k < m; ++k) {
                    double hpk = H[(size_t)p * m + k], hqk = H[(size_t)q * m + k];
                    H[(size_t)p * m + k] = c * hpk - s * hqk;
                    H[(size_t)q * m + k] = s * hpk + c * hqk;
                }
                for (int k = 0; k < m; ++k) {
                    double qkp = Q[(size_t)k * m + p], qkq = Q[(size_t)k * m + q];
                    Q[(size_t)k * m + p] = c * qkp - s * qkq;
                    Q[(size_t)k * m + q] = s * qkp + c * qkq;
                }
            }
    }
    w.resize(m);
    for (int i = 0; i < m; ++i) w[i] = H[(size_t)i * m + i];
}

struct Lanczos {
    Problem& P;
    MFSolver& S;
    const double* valsC;   // inner-product matrix
    int n, m, nev;
    double tol;
    int max_restarts;
    DevBuf<double> V, Y, w, z, rhs, partial, dh, Sbuf, tmpV;
    std::vector<double> hpart;
    int restarts = 0, op_count = 0;

    const double* valsT = nullptr;   // op = S^-1 T: T = C when null
    int rule = 0;                    // selection rule on key(theta)
    double cayley_sigma = 0.0;       // nonzero: key(theta) = 1 + 2 sigma theta (Cayley)
    bool bad_inner = false;          // the C-inner product met a non-positive norm (C not SPD)
    DevBuf<double> tv;

    Lanczos(Problem& P_, MFSolver& S_, const double* valsC_, int nev_, int m_, double tol_, int maxr)
        : P(P_), S(S_), valsC(valsC_), n(P_.nfree), m(m_), nev(nev_), tol(tol_), max_restarts(maxr) {
        tv.alloc(n);
        V.alloc((size_t)n * m);
        Y.alloc((size_t)n * m);
        tmpV.alloc((size_t)n * m);
        w.alloc(n); z.alloc(n); rhs.alloc(n);
        partial.alloc((size_t)GB * m);
        dh.alloc(m);
        Sbuf.alloc((size_t)m * m);
        hpart.resize((size_t)GB * m);
    }

    void dots(int cnt, const double* Ycols, const double* x, std::vector<double>& out) {
        int threads = 256;
        batched_dot_kernel<<<GB, threads, sizeof(double) * cnt * (threads / 32), P.stream>>>(n, cnt, Ycols, x,
                                                                                            partial.get());
        count_launch();
        KL_CUDA(cudaMemcpyAsync(hpart.data(), partial.get(), sizeof(double) * GB * cnt, cudaMemcpyDeviceToHost, P.stream));
        KL_CUDA(cudaStreamSynchronize(P.stream));
        out.assign(cnt, 0.0);
        for (int b = 0; b < GB; ++b)
            for (int i = 0; i < cnt; ++i) out[i] += hpart[(size_t)b * cnt + i];
    }

    void sub(int cnt, const double* Vcols, const std::vector<double>& h, double* x) {
        KL_CUDA(cudaMemcpyAsync(dh.get(), h.data(), sizeof(double) * cnt, cudaMemcpyHostToDevice, P.stream));
        gemv_sub_kernel<<<ceil_div(n, 256), 256, sizeof(double) * cnt, P.stream>>>(n, cnt, Vcols, dh.get(), x);
        count_launch();
    }

    double key(double th) const { return cayley_sigma != 0.0 ? 1.0 + 2.0 * cayley_sigma * th : th; }

    // indices of the Ritz values, wanted first (Spectra's selection rules on the operator values)
    std::vector<int> select_order(const std::vector<double>& theta) const {
        std::vector<int> o(theta.size());
        std::iota(o.begin(), o.end(), 0);
        auto k = [&](int i) { return key(theta[i]); };
        switch (rule) {
            case 0: std::sort(o.begin(), o.end(), [&](int a, int b) { return std::fabs(k(a)) > std::fabs(k(b)); }); break;
            case 1:
            case 3: std::sort(o.begin(), o.end(), [&](int a, int b) { return k(a) > k(b); }); break;
            case 4: std::sort(o.begin(), o.end(), [&](int a, int b) { return std::fabs(k(a)) < std::fabs(k(b)); }); break;
            case 5:
            case 7: std::sort(o.begin(), o.end(), [&](int a, int b) { return k(a) < k(b); }); break;
            case 8: {   // both ends: alternately the largest and the smallest remaining (one more from the top)
                std::vector<int> asc(o);
                std::sort(asc.begin(), asc.end(), [&](int a, int b) { return k(a) < k(b); });
                int lo = 0, hi = (int)asc.size() - 1;
                for (size_t i = 0; i < o.size(); ++i) o[i] = (i % 2 == 0) ? asc[hi--] : asc[lo++];
                break;
            }
            default: throw std::invalid_argument("selection rule must be 0, 1, 3, 4, 5, 7 or 8 for a symmetric pencil");
        }
        return o;
    }

    double* Vc(int j) { return V.get() + (size_t)j * n; }
    double* Yc(int j) { return Y.get() + (size_t)j * n; }

    // returns number of converged wanted pairs; theta/vecs of the wanted set
    int run(std::vector<double>& theta_out, std::vector<double>& S_out, std::vector<int>& sel_out) {
        std::vector<double> H((size_t)m * m, 0.0);
        // deterministic start vector
        {
            std::vector<double> v0(n);
            uint64_t st = 0x9E3779B97F4A7C15ull;
            for (int i = 0; i < n; ++i) {
                st ^= st << 13; st ^= st >> 7; st ^= st << 17;
                v0[i] = 1.0 + 0.5 * ((double)(st >> 11) / 9007199254740992.0 - 0.5);
            }
            KL_CUDA(cudaMemcpyAsync(Vc(0), v0.data(), sizeof(double) * n, cudaMemcpyHostToDevice, P.stream));
            spmv_vals(P, valsC, Vc(0), Yc(0));
            std::vector<double> d;
            dots(1, Yc(0), Vc(0), d);
            if (!(d[0] > 0.0)) {
                bad_inner = true;
                return 0;
            }
            double nr = std::sqrt(d[0]);
            vec::axpby(0.0, Vc(0), 1.0 / nr, Vc(0), n, P.stream);
            vec::axpby(0.0, Yc(0), 1.0 / nr, Yc(0), n, P.stream);
        }
        int k = 0;
        double beta_last = 0.0;
        std::vector<double> theta, Q;
        std::vector<int> order;
        for (restarts = 0;; ++restarts) {
            for (int j = k; j < m; ++j) {
                // w = op v_j = S^-1 (T v_j); with T = C the product is Y_j
                if (valsT) {
                    spmv_vals(P, valsT, Vc(j), tv.get());
                    S.solve(tv.get(), w.get(), 1);
                } else {
                    S.solve(Yc(j), w.get(), 1);
                }
                ++op_count;
                std::vector<double> h, h2;
                dots(j + 1, Y.get(), w.get(), h);
                sub(j + 1, V.get(), h, w.get());
                dots(j + 1, Y.get(), w.get(), h2);
                sub(j + 1, V.get(), h2, w.get());
                for (int i = 0; i <= j; ++i) {
                    double v = h[i] + h2[i];
                    H[(size_t)i * m + j] = v;
                    H[(size_t)j * m + i] = v;
                }
                spmv_vals(P, valsC, w.get(), z.get());
                std::vector<double> bb;
                dots(1, z.get(), w.get(), bb);
                if (bb[0] < 0.0 && -bb[0] > 1e-12 * std::fabs(H[(size_t)j * m + j])) bad_inner = true;
                double beta = std::sqrt(std::max(bb[0], 0.0));
                if (j + 1 < m) {
                    if (beta == 0.0) beta = 1e-300;
                    vec::lincomb(1.0 / beta, w.get(), 0.0, w.get(), Vc(j + 1), n, P.stream);
                    vec::lincomb(1.0 / beta, z.get(), 0.0, z.get(), Yc(j + 1), n, P.stream);
                    H[(size_t)(j + 1) * m + j] = H[(size_t)j * m + (j + 1)] = beta;
                } else {
                    beta_last = beta;
                }
            }
            jacobi_eig(m, H, theta, Q);
            order = select_order(theta);
            int nconv = 0;
            for (int i = 0; i < nev; ++i) {
                int c = order[i];
                double res = std::fabs(beta_last * Q[(size_t)(m - 1) * m + c]);
                if (res <= tol * std::max(std::fabs(theta[c]), 1e-300)) ++nconv;
            }
            if (nconv >= nev || restarts >= max_restarts) {
                theta_out = theta;
                S_out = Q;
                sel_out.assign(order.begin(), order.begin() + nev);
                return nconv;
            }
            // thick restart: keep kk Ritz vectors with the largest |theta|
            int kk = std::min(m - 1, std::max(nev + 1, nev + (m - nev) / 2));
            std::vector<double> Ssel((size_t)m * kk);
            for (int jj = 0; jj < kk; ++jj)
                for (int i = 0; i < m; ++i) Ssel[(size_t)jj * m + i] = Q[(size_t)i * m + order[jj]];
            KL_CUDA(cudaMemcpyAsync(Sbuf.get(), Ssel.data(), sizeof(double) * m * kk, cudaMemcpyHostToDevice, P.stream));
            size_t shm = sizeof(double) * m * kk;
            gemm_vs_kernel<<<ceil_div(n, 128), 128, shm, P.stream>>>(n, m, kk, V.get(), Sbuf.get(), tmpV.get());
            count_launch();
            KL_CUDA(cudaMemcpyAsync(V.get(), tmpV.get(), sizeof(double) * n * kk, cudaMemcpyDeviceToDevice, P.stream));
            gemm_vs_kernel<<<ceil_div(n, 128), 128, shm, P.stream>>>(n, m, kk, Y.get(), Sbuf.get(), tmpV.get());
            count_launch();
            KL_CUDA(cudaMemcpyAsync(Y.get(), tmpV.get(), sizeof(double) * n * kk, cudaMemcpyDeviceToDevice, P.stream));
            // next basis vector = last residual direction (w, z still hold it)
            double b = beta_last == 0.0 ? 1e-300 : beta_last;
            vec::lincomb(1.0 / b, w.get(), 0.0, w.get(), Vc(kk), n, P.stream);
            vec::lincomb(1.0 / b, z.get(), 0.0, z.get(), Yc(kk), n, P.stream);
            std::fill(H.begin(), H.end(), 0.0);
            for (int i = 0; i < kk; ++i) {
                H[(size_t)i * m + i] = theta[order[i]];
                double c = beta_last * Q[(size_t)(m - 1) * m + order[i]];
                H[(size_t)i * m + kk] = H[(size_t)kk * m + i] = c;
            }
            k = kk;
        }
    }
};

// The pencil (A, B) in operator mode `mode` (0..4, header comment), wanted operator values by
// `selection`, returned eigenvalues ordered by `sorting` (Spectra SortRule numbers).
int run_pencil(Problem& P, const Options& opt, const double* valsA, const double* valsB, int mode, int nev,
               double shift, double* values, double* vectors, int selection, int sorting) {
    int n = P.nfree;
    int64_t nnz = P.nnz;
    if (nev >= n) throw std::invalid_argument("nev must be smaller than the number of dofs");
    if (mode < 0 || mode > 4) throw std::invalid_argument("eigen solver mode must be 0..4");
    if ((mode == 3 || mode == 4) && shift == 0.0) throw std::invalid_argument("Buckling and Cayley modes need a nonzero shift");
    int ncvFac = (int)opt.integer("ncvFac", 3);
    int m = std::min<int64_t>(n, std::max<int64_t>((int64_t)ncvFac * nev, nev + 2));
    double tol = opt.real("tolerance", 1e-10);
    const bool regular = mode <= 1;
    // the factorised matrix -> d_vals64: B (regular modes) or A - sigma B
    if (regular)
        KL_CUDA(cudaMemcpyAsync(P.d_vals64.get(), valsB, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, P.stream));
    else {
        combine_kernel<<<ceil_div(nnz, 256), 256, 0, P.stream>>>(nnz, 1.0, valsA, -shift, valsB, P.d_vals64.get());
        count_launch();
    }
    if (P.d_vals32.size() < (size_t)nnz) P.d_vals32.alloc(nnz);
    // FP64 fronts by default: the FP32 factor of a large thin-shell pencil is too inaccurate for
    // iterative refinement to converge ("FrontPrecision" 32 selects FP32 fronts + refinement)
    MFSolver S(P, (int)opt.integer("Refinement", 12), opt.real("RefineTol", 1e-13),
               opt.integer("FrontPrecision", 64) == 64);
    if (S.factor_current(true) != ST_SUCCESS) return ST_SOLVER_ERROR;
    // inner-product matrix C (A for Buckling, B otherwise) and, for the regular modes, the
    // operand T = A - sigma B (copies: the inputs may alias buffers the factorisation keeps)
    DevBuf<double> valsC(nnz), valsT;
    KL_CUDA(cudaMemcpyAsync(valsC.get(), mode == 3 ? valsA : valsB, sizeof(double) * nnz, cudaMemcpyDeviceToDevice,
                            P.stream));
    if (regular) {
        valsT.alloc(nnz);
        combine_kernel<<<ceil_div(nnz, 256), 256, 0, P.stream>>>(nnz, 1.0, valsA, -shift, valsB, valsT.get());
        count_launch();
    }
    Lanczos lz(P, S, valsC.get(), nev, m, tol, (int)opt.integer("maxRestarts", 200));
    lz.valsT = regular ? valsT.get() : nullptr;
    lz.rule = selection;
    lz.cayley_sigma = mode == 4 ? shift : 0.0;
    std::vector<double> theta, Q;
    std::vector<int> sel;
    int nconv = lz.run(theta, Q, sel);
    if (lz.bad_inner) return ST_SOLVER_ERROR;   // the inner-product matrix is not positive definite
    std::vector<double> lam(nev);
    for (int i = 0; i < nev; ++i) {
        const double th = theta[sel[i]];
        lam[i] = regular ? th + shift : mode == 3 ? shift * th / (th - 1.0) : shift + 1.0 / th;
    }
    std::vector<int> idx(nev);
    std::iota(idx.begin(), idx.end(), 0);
    switch (sorting) {
        case 0: std::sort(idx.begin(), idx.end(), [&](int a, int b) { return std::fabs(lam[a]) > std::fabs(lam[b]); }); break;
        case 1:
        case 3: std::sort(idx.begin(), idx.end(), [&](int a, int b) { return lam[a] > lam[b]; }); break;
        case 4: std::sort(idx.begin(), idx.end(), [&](int a, int b) { return std::fabs(lam[a]) < std::fabs(lam[b]); }); break;
        case 5:
        case 7: std::sort(idx.begin(), idx.end(), [&](int a, int b) { return lam[a] < lam[b]; }); break;
        default: throw std::invalid_argument("sort rule must be 0, 1, 3, 4, 5 or 7 for a symmetric pencil");
    }
    for (int i = 0; i < nev; ++i) values[i] = lam[idx[i]];
    if (vectors) {
        std::vector<double> Ssel((size_t)m * nev);
        for (int j = 0; j < nev; ++j)
            for (int i = 0; i < m; ++i) Ssel[(size_t)j * m + i] = Q[(size_t)i * m + sel[idx[j]]];
        KL_CUDA(cudaMemcpyAsync(lz.Sbuf.get(), Ssel.data(), sizeof(double) * m * nev, cudaMemcpyHostToDevice, P.stream));
        gemm_vs_kernel<<<ceil_div(n, 128), 128, sizeof(double) * m * nev, P.stream>>>(n, m, nev, lz.V.get(), lz.Sbuf.get(),
                                                                                     lz.tmpV.get());
        count_launch();
        P.download_pub(lz.tmpV.get(), vectors, nev);
    }
    KL_CUDA(cudaStreamSynchronize(P.stream));
    return nconv >= nev ? ST_SUCCESS : ST_NOT_CONVERGED;
}

// the mode / rules of a call: the options when given, else the given defaults
void eigen_rules(const Options& opt, int def_mode, int& mode, int& selection, int& sorting) {
    mode = (int)opt.integer("solver", def_mode);
    selection = (int)opt.integer("selectionRule", 0);
    sorting = (int)opt.integer("sortRule", 4);
}

// ---- dense generalised eigensolver (gsEigenProblemBase::compute) --------------------------------
// Dense FP64 kernels for pencils small enough to hold as n x n matrices: B = L L^T (left-looking
// Cholesky, one column per step), C = L^-1 A L^-T (two forward substitutions, one thread per
// right-hand side), cyclic Jacobi on C with n/2 disjoint rotations per round (round-robin pairing,
// a grid-wide barrier between the rotation, row and column phases), x = L^-T V.

// D[i * n + j] = A(i, j) (row-major dense copy of CSR values)
__global__ void csr_to_dense_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ cols,
                                    const double* __restrict__ vals, double* __restrict__ D) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) D[(size_t)r * n + cols[k]] = vals[k];
}

// Cholesky column j of the lower factor L (row-major, overwrites the lower triangle of B):
// step 1 t(i) = B(i, j) - sum_{k<j} L(i, k) L(j, k) for i >= j; step 2 L(j, j) = sqrt(t(j)),
// L(i, j) = t(i) / L(j, j).  A non-positive pivot sets *status.
__global__ void chol_col_dot_kernel(int n, int j, const double* __restrict__ L, double* __restrict__ t) {
    int i = j + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* li = L + (size_t)i * n;
    const double* lj = L + (size_t)j * n;
    double s = li[j];
    for (int k = 0; k < j; ++k) s -= li[k] * lj[k];
    t[i] = s;
}
__global__ void chol_col_scale_kernel(int n, int j, double* __restrict__ L, const double* __restrict__ t, int* status) {
    int i = j + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = t[j];
    if (!(d > 0.0)) {
        if (i == j) atomicExch(status, 1);
        return;
    }
    const double ljj = sqrt(d);
    L[(size_t)i * n + j] = i == j ? ljj : t[i] / ljj;
}

// X <- L^-1 X (forward substitution), X row-major n x n, one thread per column
__global__ void lower_solve_kernel(int n, const double* __restrict__ L, double* __restrict__ X) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    for (int i = 0; i < n; ++i) {
        const double* li = L + (size_t)i * n;
        double s = X[(size_t)i * n + c];
        for (int k = 0; k < i; ++k) s -= li[k] * X[(size_t)k * n + c];
        X[(size_t)i * n + c] = s / li[i];
    }
}
// X <- L^-T X (backward substitution)
__global__ void upper_solve_kernel(int n, const double* __restrict__ L, double* __restrict__ X) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    for (int i = n - 1; i >= 0; --i) {
        double s = X[(size_t)i * n + c];
        for (int k = i + 1; k < n; ++k) s -= L[(size_t)k * n + i] * X[(size_t)k * n + c];
        X[(size_t)i * n + c] = s / L[(size_t)i * n + i];
    }
}
// Y = (X + X^T) / 2 written transposed-safe: Y(i, j) for i <= j and its mirror
__global__ void transpose_kernel(int n, const double* __restrict__ X, double* __restrict__ Y) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= (int64_t)n * n) return;
    const int i = (int)(e / n), j = (int)(e % n);
    Y[(size_t)j * n + i] = X[e];
}
__global__ void symmetrize_kernel(int n, double* __restrict__ C) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= (int64_t)n * n) return;
    const int i = (int)(e / n), j = (int)(e % n);
    if (i < j) {
        const double v = 0.5 * (C[e] + C[(size_t)j * n + i]);
        C[e] = v;
        C[(size_t)j * n + i] = v;
    }
}

// player at seat j (1..N-1) of round r in the circle schedule; seat 0 holds player 0
__device__ __forceinline__ int rr_seat(int j, int r, int N) { return j == 0 ? 0 : ((j - 1 + r) % (N - 1)) + 1; }

// Cyclic Jacobi on the symmetric row-major C (n x n), eigenvectors accumulated in the row-major V
// (columns).  Stops when the off-diagonal mass is below tol2 of the total or after max_sweeps.
__global__ void __launch_bounds__(256) dense_jacobi_kernel(int n, double* __restrict__ C, double* __restrict__ V,
                                                          double* __restrict__ rot, double* __restrict__ red,
                                                          int max_sweeps, double tol2, int* sweeps_done) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    __shared__ double sred[2][8];
    const int N = n + (n & 1);                  // even number of players (player n is a bye)
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        // off-diagonal and total squared mass (every block sums the partials itself)
        double off = 0.0, tot = 0.0;
        for (int64_t e = tid; e < (int64_t)n * n; e += nthr) {
            const double v = C[e] * C[e];
            tot += v;
            if (e / n != e % n) off += v;
        }
        for (int o = 16; o > 0; o >>= 1) {
            off += __shfl_xor_sync(0xffffffffu, off, o);
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
        }
        if (lane == 0) { sred[0][warp] = off; sred[1][warp] = tot; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double a = 0.0, b = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { a += sred[0][w]; b += sred[1][w]; }
            red[2 * blockIdx.x] = a;
            red[2 * blockIdx.x + 1] = b;
        }
        grid.sync();
        double OFF = 0.0, TOT = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b) { OFF += red[2 * b]; TOT += red[2 * b + 1]; }
        if (OFF <= tol2 * TOT || OFF == 0.0) break;
        for (int r = 0; r < N - 1; ++r) {
            // rotations of the round's pairs
            for (int64_t t = tid; t < N / 2; t += nthr) {
                int p = rr_seat((int)t, r, N), q = rr_seat(N - 1 - (int)t, r, N);
                if (p > q) { const int x = p; p = q; q = x; }
                double c = 1.0, s = 0.0;
                if (q < n) {
                    const double apq = C[(size_t)p * n + q];
                    if (fabs(apq) > 1e-300) {
                        const double app = C[(size_t)p * n + p], aqq = C[(size_t)q * n + q];
                        const double theta = (aqq - app) / (2.0 * apq);
                        const double tt = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                        c = 1.0 / sqrt(tt * tt + 1.0);
                        s = tt * c;
                    }
                }
                rot[4 * t] = p; rot[4 * t + 1] = q; rot[4 * t + 2] = c; rot[4 * t + 3] = s;
            }
            grid.sync();
            // rows p, q of C
            for (int64_t e = tid; e < (int64_t)(N / 2) * n; e += nthr) {
                const int t = (int)(e / n), k = (int)(e % n);
                const int p = (int)rot[4 * t], q = (int)rot[4 * t + 1];
                if (q >= n) continue;
                const double c = rot[4 * t + 2], s = rot[4 * t + 3];
                const double a = C[(size_t)p * n + k], b = C[(size_t)q * n + k];
                C[(size_t)p * n + k] = c * a - s * b;
                C[(size_t)q * n + k] = s * a + c * b;
            }
            grid.sync();
            // columns p, q of C and of V
            for (int64_t e = tid; e < (int64_t)(N / 2) * n; e += nthr) {
                const int t = (int)(e / n), k = (int)(e % n);
                const int p = (int)rot[4 * t], q = (int)rot[4 * t + 1];
                if (q >= n) continue;
                const double c = rot[4 * t + 2], s = rot[4 * t + 3];
                double a = C[(size_t)k * n + p], b = C[(size_t)k * n + q];
                C[(size_t)k * n + p] = c * a - s * b;
                C[(size_t)k * n + q] = s * a + c * b;
                a = V[(size_t)k * n + p];
                b = V[(size_t)k * n + q];
                V[(size_t)k * n + p] = c * a - s * b;
                V[(size_t)k * n + q] = s * a + c * b;
            }
            grid.sync();
        }
    }
    if (tid == 0) *sweeps_done = sweep;
}

__global__ void identity_dense_kernel(int n, double* __restrict__ V) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e < (int64_t)n * n) V[e] = (e / n == e % n) ? 1.0 : 0.0;
}

// The pencil of an eigen problem on the device, FP64 values on the problem's CSR pattern:
// kind 0 gsModalSolver (A = K at zero, B = M); kind 1 gsBucklingSolver (gsBucklingSolver.h:127-149:
// u_L = K_L^-1 (scaling F), A = K_L, B = K(u_L) - K_L).
int assemble_pencil(Problem& P, const Options& opt, int kind, double scaling, DevBuf<double>& A, DevBuf<double>& B) {
    const int n = P.nfree;
    const int64_t nnz = P.nnz;
    A.alloc(nnz);
    B.alloc(nnz);
    DevBuf<double> z(n);
    z.zero(P.stream);
    P.set_displacement(z.get());
    P.tangent_f64();
    KL_CUDA(cudaMemcpyAsync(A.get(), P.d_vals64.get(), sizeof(double) * nnz, cudaMemcpyDeviceToDevice, P.stream));
    if (kind == 0) {
        P.mass_f64();
        KL_CUDA(cudaMemcpyAsync(B.get(), P.d_vals64.get(), sizeof(double) * nnz, cudaMemcpyDeviceToDevice, P.stream));
        return ST_SUCCESS;
    }
    if (kind != 1) throw std::invalid_argument("eigen problem kind must be 0 (modal) or 1 (buckling)");
    DevBuf<double> uL(n), rhs(n);
    {
        MFSolver S(P, (int)opt.integer("Refinement", 12), opt.real("RefineTol", 1e-13),
                   opt.integer("FrontPrecision", 64) == 64);
        if (S.factor_current(true) != ST_SUCCESS) return ST_SOLVER_ERROR;
        vec::lincomb(scaling, P.d_F.get(), 0.0, P.d_F.get(), rhs.get(), n, P.stream);
        S.solve(rhs.get(), uL.get(), 1);
    }
    P.set_displacement(uL.get());
    P.tangent_f64();
    combine_kernel<<<ceil_div(nnz, 256), 256, 0, P.stream>>>(nnz, 1.0, P.d_vals64.get(), -1.0, A.get(), B.get());
    count_launch();
    return ST_SUCCESS;
}

}  // namespace

void spmv_vals(const Problem& P, const double* vals, const double* x, double* y) {
    spmv_vals_kernel<<<ceil_div((int64_t)P.nfree * 32, 256), 256, 0, P.stream>>>(P.nfree, P.d_rowptr.get(), P.d_cols.get(),
                                                                                 vals, x, y);
    count_launch();
}

int buckling_gpu(Problem& P, const Options& opt, int nev, double shift, double scaling, double* values, double* vectors) {
    int n = P.nfree;
    int64_t nnz = P.nnz;
    DevBuf<double> KL(nnz), B(nnz), uL(n), rhs(n);
    // K_L at u = 0 (FP64), u_L = K_L^-1 (s F) with refinement
    rhs.zero(P.stream);
    P.set_displacement(rhs.get());
    P.tangent_f64();
    KL_CUDA(cudaMemcpyAsync(KL.get(), P.d_vals64.get(), sizeof(double) * nnz, cudaMemcpyDeviceToDevice, P.stream));
    {
        MFSolver S(P, (int)opt.integer("Refinement", 12), opt.real("RefineTol", 1e-13),
                   opt.integer("FrontPrecision", 64) == 64);
        if (S.factor_current(true) != ST_SUCCESS) return ST_SOLVER_ERROR;
        vec::lincomb(scaling, P.d_F.get(), 0.0, P.d_F.get(), rhs.get(), n, P.stream);
        S.solve(rhs.get(), uL.get(), 1);
    }
    P.set_displacement(uL.get());
    P.tangent_f64();
    combine_kernel<<<ceil_div(nnz, 256), 256, 0, P.stream>>>(nnz, 1.0, P.d_vals64.get(), -1.0, KL.get(), B.get());
    count_launch();
    int mode, selection, sorting;
    eigen_rules(opt, 3, mode, selection, sorting);
    return run_pencil(P, opt, KL.get(), B.get(), mode, nev, shift, values, vectors, selection, sorting);
}

int standard_eigs_gpu(Problem& P, const double* valsA, int nev, int ncv_fac, double shift, double tol, double* values) {
    int64_t nnz = P.nnz;
    DevBuf<double> A(nnz), I(nnz);
    KL_CUDA(cudaMemcpyAsync(A.get(), valsA, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, P.stream));
    identity_vals_kernel<<<ceil_div(P.nfree, 256), 256, 0, P.stream>>>(P.nfree, P.d_rowptr.get(), P.d_cols.get(), I.get());
    count_launch();
    Options o;
    o.ints["ncvFac"] = ncv_fac;
    o.reals["tolerance"] = tol;
    o.ints["maxRestarts"] = 1000;
    return run_pencil(P, o, A.get(), I.get(), 2, nev, shift, values, nullptr, 3, 7);
}

int modal_gpu(Problem& P, const Options& opt, int nev, double shift, double* values, double* vectors) {
    int n = P.nfree;
    int64_t nnz = P.nnz;
    DevBuf<double> K(nnz), M(nnz), z(n);
    z.zero(P.stream);
    P.set_displacement(z.get());
    P.tangent_f64();
    KL_CUDA(cudaMemcpyAsync(K.get(), P.d_vals64.get(), sizeof(double) * nnz, cudaMemcpyDeviceToDevice, P.stream));
    P.mass_f64();
    KL_CUDA(cudaMemcpyAsync(M.get(), P.d_vals64.get(), sizeof(double) * nnz, cudaMemcpyDeviceToDevice, P.stream));
    int mode, selection, sorting;
    eigen_rules(opt, 2, mode, selection, sorting);
    return run_pencil(P, opt, K.get(), M.get(), mode, nev, shift, values, vectors, selection, sorting);
}

// gsEigenProblemBase::computePower (gsEigenProblemBase.hpp:218-258): power iteration on
// D = A^-1 B from the all-ones vector, v <- D v / |D v|, until |v - v_old| < tolerance (at most 100
// steps, NotConverged after the last), value = (v.v) / (v.D v).  The reference forms A^-1 densely;
// here every product with A^-1 is a solve with the FP64 multifrontal factor of A, so the iterates
// are the same to rounding and the method scales to sparse sizes.
int power_gpu(Problem& P, const Options& opt, int kind, double scaling, double* value, double* vector) {
    const int n = P.nfree;
    const int64_t nnz = P.nnz;
    DevBuf<double> A, B;
    int st = assemble_pencil(P, opt, kind, scaling, A, B);
    if (st != ST_SUCCESS) return st;
    KL_CUDA(cudaMemcpyAsync(P.d_vals64.get(), A.get(), sizeof(double) * nnz, cudaMemcpyDeviceToDevice, P.stream));
    if (P.d_vals32.size() < (size_t)nnz) P.d_vals32.alloc(nnz);
    MFSolver S(P, (int)opt.integer("Refinement", 12), opt.real("RefineTol", 1e-13),
               opt.integer("FrontPrecision", 64) == 64);
    if (S.factor_current(true) != ST_SUCCESS) return ST_SOLVER_ERROR;
    const double tol = opt.real("tolerance", 1e-10);
    const int kmax = 100;
    DevBuf<double> v(n), vold(n), t(n), diff(n);
    std::vector<double> ones(n, 1.0);
    KL_CUDA(cudaMemcpyAsync(v.get(), ones.data(), sizeof(double) * n, cudaMemcpyHostToDevice, P.stream));
    vold.zero(P.stream);
    st = ST_NOT_CONVERGED;
    for (int k = 0; k != kmax; ++k) {
        spmv_vals(P, B.get(), v.get(), t.get());
        S.solve(t.get(), v.get(), 1);                      // v = D v
        double nn;
        const double* a1[1] = {v.get()};
        vec::multidot(1, a1, a1, n, &nn, P.stream);
        vec::axpby(0.0, v.get(), 1.0 / std::sqrt(nn), v.get(), n, P.stream);   // v.normalize()
        vec::lincomb(1.0, v.get(), -1.0, vold.get(), diff.get(), n, P.stream);
        double e2;
        const double* a2[1] = {diff.get()};
        vec::multidot(1, a2, a2, n, &e2, P.stream);
        if (std::sqrt(e2) < tol) {
            st = ST_SUCCESS;
            break;
        }
        KL_CUDA(cudaMemcpyAsync(vold.get(), v.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice, P.stream));
    }
    // value = (v.v) / (v.D v)
    spmv_vals(P, B.get(), v.get(), t.get());
    S.solve(t.get(), diff.get(), 1);
    double d[2];
    const double* xs[2] = {v.get(), v.get()};
    const double* ys[2] = {v.get(), diff.get()};
    vec::multidot(2, xs, ys, n, d, P.stream);
    *value = d[0] / d[1];
    if (vector) P.download_pub(v.get(), vector, 1);
    KL_CUDA(cudaStreamSynchronize(P.stream));
    return st;
}

// gsEigenProblemBase::compute (gsEigenProblemBase.hpp:21-50): every eigenpair of the dense
// pencil (A - shift B, B), eigenvalues + shift ascending, eigenvectors B-normalised (x^T B x = 1),
// as Eigen's GeneralizedSelfAdjointEigenSolver returns them.  B must be positive definite (a
// non-positive Cholesky pivot gives SolverError).  n x n FP64 on the device: for dense-sized
// pencils only (the caller limits n).
int dense_gpu(Problem& P, const Options& opt, int kind, double scaling, double* values, double* vectors) {
    const int n = P.nfree;
    const int64_t nnz = P.nnz;
    DevBuf<double> A, B;
    int st = assemble_pencil(P, opt, kind, scaling, A, B);
    if (st != ST_SUCCESS) return st;
    const double shift = opt.real("shift", 0.0);
    if (shift != 0.0) {   // A - shift B
        combine_kernel<<<ceil_div(nnz, 256), 256, 0, P.stream>>>(nnz, 1.0, A.get(), -shift, B.get(), A.get());
        count_launch();
    }
    const size_t nn = (size_t)n * n;
    DevBuf<double> Ad(nn), L(nn), X(nn), V(nn), t(n);
    DevBuf<int> status(1);
    Ad.zero(P.stream);
    L.zero(P.stream);
    status.zero(P.stream);
    csr_to_dense_kernel<<<ceil_div(n, 128), 128, 0, P.stream>>>(n, P.d_rowptr.get(), P.d_cols.get(), A.get(), Ad.get());
    csr_to_dense_kernel<<<ceil_div(n, 128), 128, 0, P.stream>>>(n, P.d_rowptr.get(), P.d_cols.get(), B.get(), L.get());
    count_launch(2);
    for (int j = 0; j < n; ++j) {
        chol_col_dot_kernel<<<ceil_div(n - j, 128), 128, 0, P.stream>>>(n, j, L.get(), t.get());
        chol_col_scale_kernel<<<ceil_div(n - j, 128), 128, 0, P.stream>>>(n, j, L.get(), t.get(), status.get());
        count_launch(2);
    }
    int hst = 0;
    KL_CUDA(cudaMemcpyAsync(&hst, status.get(), sizeof(int), cudaMemcpyDeviceToHost, P.stream));
    KL_CUDA(cudaStreamSynchronize(P.stream));
    if (hst) return ST_SOLVER_ERROR;
    // C = L^-1 A L^-T: X = L^-1 A, then C = L^-1 X^T (A symmetric)
    lower_solve_kernel<<<ceil_div(n, 64), 64, 0, P.stream>>>(n, L.get(), Ad.get());
    transpose_kernel<<<ceil_div((int64_t)nn, 256), 256, 0, P.stream>>>(n, Ad.get(), X.get());
    lower_solve_kernel<<<ceil_div(n, 64), 64, 0, P.stream>>>(n, L.get(), X.get());
    symmetrize_kernel<<<ceil_div((int64_t)nn, 256), 256, 0, P.stream>>>(n, X.get());
    identity_dense_kernel<<<ceil_div((int64_t)nn, 256), 256, 0, P.stream>>>(n, V.get());
    count_launch(5);
    // Jacobi: one cooperative launch, a CTA set resident on every SM
    int dev = 0, sms = 0, bps = 0;
    KL_CUDA(cudaGetDevice(&dev));
    KL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    KL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, dense_jacobi_kernel, 256, 0));
    const int grid = std::max(1, std::min(sms * std::min(bps, 2), ceil_div((int64_t)nn, 256)));
    DevBuf<double> rot((size_t)4 * (n / 2 + 1)), red((size_t)2 * grid);
    DevBuf<int> sweeps(1);
    int nval = n, maxsw = (int)opt.integer("maxSweeps", 60);
    double tol2 = 1e-30;
    double* Xp = X.get();
    double* Vp = V.get();
    double* rotp = rot.get();
    double* redp = red.get();
    int* swp = sweeps.get();
    void* args[] = {&nval, &Xp, &Vp, &rotp, &redp, &maxsw, &tol2, &swp};
    KL_CUDA(cudaLaunchCooperativeKernel((const void*)dense_jacobi_kernel, dim3(grid), dim3(256), args, 0, P.stream));
    count_launch();
    // x = L^-T V
    upper_solve_kernel<<<ceil_div(n, 64), 64, 0, P.stream>>>(n, L.get(), V.get());
    count_launch();
    std::vector<double> C(nn), Vh(nn);
    int hsw = 0;
    KL_CUDA(cudaMemcpyAsync(C.data(), X.get(), sizeof(double) * nn, cudaMemcpyDeviceToHost, P.stream));
    KL_CUDA(cudaMemcpyAsync(Vh.data(), V.get(), sizeof(double) * nn, cudaMemcpyDeviceToHost, P.stream));
    KL_CUDA(cudaMemcpyAsync(&hsw, sweeps.get(), sizeof(int), cudaMemcpyDeviceToHost, P.stream));
    KL_CUDA(cudaStreamSynchronize(P.stream));
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return C[(size_t)a * n + a] < C[(size_t)b * n + b]; });
    for (int j = 0; j < n; ++j) values[j] = C[(size_t)idx[j] * n + idx[j]] + shift;
    if (vectors) {
        // column idx[j] of V (internal order) -> row j of the output (public order)
        std::vector<double> cols(nn);
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) cols[(size_t)j * n + i] = Vh[(size_t)i * n + idx[j]];
        DevBuf<double> dv(nn);
        dv.upload(cols, P.stream);
        P.download_pub(dv.get(), vectors, n);
        KL_CUDA(cudaStreamSynchronize(P.stream));
    }
    return hsw < maxsw ? ST_SUCCESS : ST_NOT_CONVERGED;
}

}  // namespace klsa
