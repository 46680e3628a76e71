// predictor.cu -- learned arc-length predictor (no counterpart in the reference, which offers
// only the setInitialGuess hook, gsALMSolvers/gsALMBase.h:184).
//
// Features (132 = 4 x (32 + 1)) of the last four converged points P_k..P_{k-3}:
//   [q_k, L_k,  q_{k-1} - q_k, L_{k-1} - L_k,  q_{k-2} - q_k, ...,  q_{k-3} - q_k, ...],
// q = Phi^T U (Phi: orthonormal reduced modal basis), standardised with the training means and
// standard deviations.  The network output (33) is the standardised correction of the cubic
// extrapolation P_ext = 4 P_k - 6 P_{k-1} + 4 P_{k-2} - P_{k-3} inside the modal subspace:
//   U_guess = U_ext + Phi dq,   L_guess = L_ext + dL.
// Without a network (net == null) the guess is the plain cubic extrapolation.
#include "predictor.h"

#include <cmath>
#include <stdexcept>

namespace klsa {

namespace {

constexpr int PB = 152;   // blocks of the projection kernel

__global__ void project_kernel(int n, int nm, const double* __restrict__ Phi, const double* __restrict__ u,
                               double* __restrict__ partial) {
    extern __shared__ double red[];   // nm * (blockDim / 32)
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = 0; j < nm; ++j) {
        double s = 0.0;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            s += Phi[(size_t)j * n + i] * u[i];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) red[j * nw + warp] = s;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nm; j += blockDim.x) {
        double s = 0.0;
        for (int w = 0; w < nw; ++w) s += red[j * nw + w];
        partial[(size_t)blockIdx.x * nm + j] = s;
    }
}

__global__ void guess_kernel(int n, int nm, const double* __restrict__ h0, const double* __restrict__ h1,
                             const double* __restrict__ h2, const double* __restrict__ h3,
                             const double* __restrict__ Phi, const double* __restrict__ dq, double* __restrict__ Ug) {
    extern __shared__ double q[];
    for (int j = threadIdx.x; j < nm; j += blockDim.x) q[j] = dq[j];
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = 4.0 * h0[i] - 6.0 * h1[i] + 4.0 * h2[i] - h3[i];
    for (int j = 0; j < nm; ++j) v += Phi[(size_t)j * n + i] * q[j];
    Ug[i] = v;
}

}  // namespace

LearnedPredictor::LearnedPredictor(Problem& P_, MLP* net_, const double* modes_pub, int nm_, const double* imu,
                                   const double* isd, const double* omu, const double* osd)
    : P(P_), net(net_), nm(nm_) {
    int n = P.nfree;
    if (nm < 0 || nm > 256) throw std::invalid_argument("number of modes must be in 0..256");
    if (net && (net->in != 4 * (nm + 1) || net->out != nm + 1))
        throw std::invalid_argument("network shape must be in = 4 (modes + 1), out = modes + 1");
    Phi.alloc((size_t)std::max(nm, 1) * n);
    if (nm > 0) {
        DevBuf<double> tmp((size_t)nm * n);
        KL_CUDA(cudaMemcpyAsync(tmp.get(), modes_pub, sizeof(double) * nm * n, cudaMemcpyHostToDevice, P.stream));
        P.pub_to_int(tmp.get(), Phi.get(), nm);
        KL_CUDA(cudaStreamSynchronize(P.stream));
    }
    int nin = 4 * (nm + 1), nout = nm + 1;
    in_mu.assign(imu ? imu : nullptr, imu ? imu + nin : nullptr);
    in_sd.assign(isd ? isd : nullptr, isd ? isd + nin : nullptr);
    out_mu.assign(omu ? omu : nullptr, omu ? omu + nout : nullptr);
    out_sd.assign(osd ? osd : nullptr, osd ? osd + nout : nullptr);
    if (in_mu.empty()) in_mu.assign(nin, 0.0);
    if (in_sd.empty()) in_sd.assign(nin, 1.0);
    if (out_mu.empty()) out_mu.assign(nout, 0.0);
    if (out_sd.empty()) out_sd.assign(nout, 1.0);
    hist.alloc((size_t)4 * n);
    histq.assign((size_t)4 * std::max(nm, 1), 0.0);
    dq.alloc(std::max(nm, 1));
    part.alloc((size_t)PB * std::max(nm, 1));
    feat.alloc(nin);
    hpart.resize((size_t)PB * std::max(nm, 1));
}

void LearnedPredictor::project(const double* dU, double* q) {
    if (nm == 0) return;
    int threads = 256;
    project_kernel<<<PB, threads, sizeof(double) * nm * (threads / 32), P.stream>>>(P.nfree, nm, Phi.get(), dU,
                                                                                   part.get());
    count_launch();
    KL_CUDA(cudaMemcpyAsync(hpart.data(), part.get(), sizeof(double) * PB * nm, cudaMemcpyDeviceToHost, P.stream));
    KL_CUDA(cudaStreamSynchronize(P.stream));
    for (int j = 0; j < nm; ++j) {
        double s = 0.0;
        for (int b = 0; b < PB; ++b) s += hpart[(size_t)b * nm + j];
        q[j] = s;
    }
}

void LearnedPredictor::push(const double* dU, double L) {
    int n = P.nfree;
    KL_CUDA(cudaMemcpyAsync(hist.get() + (size_t)head * n, dU, sizeof(double) * n, cudaMemcpyDeviceToDevice, P.stream));
    histL[head] = L;
    project(dU, histq.data() + (size_t)head * std::max(nm, 1));
    head = (head + 1) & 3;
    count = std::min(count + 1, 4);
}

bool LearnedPredictor::guess(double* dUg, double* Lg) {
    if (count < 4) return false;
    int n = P.nfree, s0 = slot(0), s1 = slot(1), s2 = slot(2), s3 = slot(3);
    const int M = std::max(nm, 1);
    const double* q0 = histq.data() + (size_t)s0 * M;
    const double* qs[4] = {q0, histq.data() + (size_t)s1 * M, histq.data() + (size_t)s2 * M,
                           histq.data() + (size_t)s3 * M};
    const double Ls[4] = {histL[s0], histL[s1], histL[s2], histL[s3]};
    std::vector<double> corr(nm + 1, 0.0);
    if (net) {
        int nin = 4 * (nm + 1);
        std::vector<float> f(nin);
        for (int b = 0; b < 4; ++b) {
            for (int j = 0; j < nm; ++j) {
                double v = (b == 0) ? q0[j] : qs[b][j] - q0[j];
                int idx = b * (nm + 1) + j;
                f[idx] = (float)((v - in_mu[idx]) / in_sd[idx]);
            }
            double vl = (b == 0) ? Ls[0] : Ls[b] - Ls[0];
            int idx = b * (nm + 1) + nm;
            f[idx] = (float)((vl - in_mu[idx]) / in_sd[idx]);
        }
        feat.upload(f, net->stream);
        net->forward(feat.get(), 1);
        std::vector<float> y(nm + 1);
        KL_CUDA(cudaMemcpyAsync(y.data(), net->Y.get(), sizeof(float) * (nm + 1), cudaMemcpyDeviceToHost, net->stream));
        KL_CUDA(cudaStreamSynchronize(net->stream));
        for (int j = 0; j <= nm; ++j) corr[j] = y[j] * out_sd[j] + out_mu[j];
    }
    if (nm > 0) KL_CUDA(cudaMemcpyAsync(dq.get(), corr.data(), sizeof(double) * nm, cudaMemcpyHostToDevice, P.stream));
    const double* H = hist.get();
    guess_kernel<<<ceil_div(n, 256), 256, sizeof(double) * M, P.stream>>>(
        n, nm, H + (size_t)s0 * n, H + (size_t)s1 * n, H + (size_t)s2 * n, H + (size_t)s3 * n, Phi.get(), dq.get(), dUg);
    count_launch();
    KL_CHECK_LAUNCH();
    *Lg = 4.0 * Ls[0] - 6.0 * Ls[1] + 4.0 * Ls[2] - Ls[3] + corr[nm];
    return true;
}

}  // namespace klsa
