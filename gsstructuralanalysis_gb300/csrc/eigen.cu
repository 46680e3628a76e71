// eigen.cu -- thick-restart shift-invert Lanczos with FP64 full reorthogonalisation.
//
// Generalised symmetric pencil A v = lambda B v, operator op = (A - sigma B)^-1 C with the
// C-inner product:
//   ShiftInvert (modal, B SPD):      C = B, op eigenvalue nu = 1/(lambda - sigma)
//   Buckling    (A SPD, B indefinite): C = A, nu = lambda/(lambda - sigma)
// (the two Spectra GEigsMode variants the reference selects, gsEigenProblemBase.hpp:152-215).
// (A - sigma B) is factorised once by the multifrontal LDL^T in FP32; every application of op
// is polished by FP64 iterative refinement against the FP64 CSR values.  The Lanczos basis V
// and its image Y = C V stay in HBM (FP64); reorthogonalisation is classical Gram-Schmidt done
// twice with batched dot products; the small projected matrix is diagonalised on the host by
// cyclic Jacobi in FP64.
#include "eigen.h"

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

    bool largest_alge = false;   // wanted Ritz values: largest |theta| (false) or largest theta (true)

    Lanczos(Problem& P_, MFSolver& S_, const double* valsC_, int nev_, int m_, double tol_, int maxr)
        : P(P_), S(S_), valsC(valsC_), n(P_.nfree), m(m_), nev(nev_), tol(tol_), max_restarts(maxr) {
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
                // w = op v_j = (A - sigma B)^-1 (C v_j) = solve(Y_j)
                S.solve(Yc(j), w.get(), 1);
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
            order.resize(m);
            std::iota(order.begin(), order.end(), 0);
            if (largest_alge)
                std::sort(order.begin(), order.end(), [&](int a, int b) { return theta[a] > theta[b]; });
            else
                std::sort(order.begin(), order.end(), [&](int a, int b) { return std::fabs(theta[a]) > std::fabs(theta[b]); });
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

// largest_alge: select the largest transformed values nu (Spectra LargestAlge) instead of the
// largest |nu| (LargestMagn); sort_alge: return the eigenvalues ascending (SmallestAlge) instead
// of by ascending |lambda| (SmallestMagn).
int run_pencil(Problem& P, const Options& opt, const double* valsA, const double* valsB, bool buckling_mode, int nev,
               double shift, double* values, double* vectors, bool largest_alge = false, bool sort_alge = false) {
    int n = P.nfree;
    int64_t nnz = P.nnz;
    if (nev >= n) throw std::invalid_argument("nev must be smaller than the number of dofs");
    int ncvFac = (int)opt.integer("ncvFac", 3);
    int m = std::min<int64_t>(n, std::max<int64_t>((int64_t)ncvFac * nev, nev + 2));
    double tol = opt.real("tolerance", 1e-10);
    // op matrix (A - sigma B) -> d_vals64, factorised in FP32, refined in FP64
    combine_kernel<<<ceil_div(nnz, 256), 256, 0, P.stream>>>(nnz, 1.0, valsA, -shift, valsB, P.d_vals64.get());
    count_launch();
    if (P.d_vals32.size() < (size_t)nnz) P.d_vals32.alloc(nnz);
    // FP64 fronts by default: the FP32 factor of a large thin-shell pencil is too inaccurate for
    // iterative refinement to converge ("FrontPrecision" 32 selects FP32 fronts + refinement)
    MFSolver S(P, (int)opt.integer("Refinement", 12), opt.real("RefineTol", 1e-13),
               opt.integer("FrontPrecision", 64) == 64);
    if (S.factor_current(true) != ST_SUCCESS) return ST_SOLVER_ERROR;
    // copy C values (they may alias a scratch buffer that the factorisation keeps)
    DevBuf<double> valsC(nnz);
    KL_CUDA(cudaMemcpyAsync(valsC.get(), buckling_mode ? valsA : valsB, sizeof(double) * nnz, cudaMemcpyDeviceToDevice,
                            P.stream));
    Lanczos lz(P, S, valsC.get(), nev, m, tol, (int)opt.integer("maxRestarts", 200));
    lz.largest_alge = largest_alge;
    std::vector<double> theta, Q;
    std::vector<int> sel;
    int nconv = lz.run(theta, Q, sel);
    // transform back and sort by |lambda| ascending (sortRule SmallestMagn)
    std::vector<double> lam(nev);
    for (int i = 0; i < nev; ++i) {
        double th = theta[sel[i]];
        lam[i] = buckling_mode ? shift * th / (th - 1.0) : shift + 1.0 / th;
    }
    std::vector<int> idx(nev);
    std::iota(idx.begin(), idx.end(), 0);
    if (sort_alge)
        std::sort(idx.begin(), idx.end(), [&](int a, int b) { return lam[a] < lam[b]; });
    else
        std::sort(idx.begin(), idx.end(), [&](int a, int b) { return std::fabs(lam[a]) < std::fabs(lam[b]); });
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

}  // namespace

void spmv_vals(const Problem& P, const double* vals, const double* x, double* y) {
    spmv_vals_kernel<<<ceil_div((int64_t)P.nfree * 32, 256), 256, 0, P.stream>>>(P.nfree, P.d_rowptr.get(), P.d_cols.get(),
                                                                                 vals, x, y);
    count_launch();
}

int buckling_gpu(Problem& P, const Options& opt, int nev, double shift, double scaling, double* values, double* vectors) {
    if (shift == 0.0) throw std::invalid_argument("buckling mode needs a nonzero shift");
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
    return run_pencil(P, opt, KL.get(), B.get(), true, nev, shift, values, vectors);
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
    return run_pencil(P, o, A.get(), I.get(), false, nev, shift, values, nullptr, true, true);
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
    return run_pencil(P, opt, K.get(), M.get(), false, nev, shift, values, vectors);
}

}  // namespace klsa
