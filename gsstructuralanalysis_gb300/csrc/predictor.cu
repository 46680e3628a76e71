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

constexpr int PCH = LearnedPredictor::PCH;

// qslot[c * nm + j] = sum over chunk c of Phi_j . u (fixed order within the chunk)
__global__ void __launch_bounds__(256) project_kernel(int n, int nm, const double* __restrict__ Phi,
                                                      const double* __restrict__ u, double* __restrict__ qslot) {
    __shared__ double red[8];
    const int j = blockIdx.y, c = blockIdx.x;
    const int len = (n + PCH - 1) / PCH, lo = c * len, hi = min(n, lo + len);
    const double* ph = Phi + (size_t)j * n;
    double s = 0.0;
#pragma unroll 4
    for (int i = lo + threadIdx.x; i < hi; i += 256) s += ph[i] * u[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += red[w];
        qslot[(size_t)c * nm + j] = t;
    }
}

struct InferArgs {
    const double* qpart;   // ring of 4 slots, PCH x nm each
    int slot[4];           // newest first
    double L[4];
    int nm, in, h1, h2, out;
    const double* stats;   // in_mu[in] in_sd[in] out_mu[out] out_sd[out]
    const float *W1, *b1, *W2, *b2, *W3, *b3;
    double* corr;          // out: destandardised network output
};

// one dense layer of the network for one input row: warp w owns outputs w, w + nwarps, ...; the
// lanes read a weight row in consecutive 128-byte pieces and the warp sums their products
template <bool GELU>
__device__ __forceinline__ void dense_warp_layer(int nout, int nin, const float* __restrict__ W,
                                                 const float* __restrict__ b, const float* x, float* y) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int r = warp; r < nout; r += nw) {
        const float* w = W + (size_t)r * nin;
        float acc = 0.f;
        for (int k = lane; k < nin; k += 32) acc = fmaf(x[k], w[k], acc);
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            acc += b[r];
            if (GELU) acc = 0.5f * acc * (1.f + erff(acc * 0.70710678118654752f));
            y[r] = acc;
        }
    }
}

// features of the last four points -> network -> corr (one CTA of 32 warps; the weights stay in L2)
__global__ void __launch_bounds__(1024) infer_kernel(InferArgs a) {
    extern __shared__ float sm[];
    float* x = sm;
    float* y1 = x + a.in;
    float* y2 = y1 + a.h1;
    const int M1 = a.nm + 1;
    const double *in_mu = a.stats, *in_sd = a.stats + a.in, *out_mu = a.stats + 2 * a.in,
                 *out_sd = a.stats + 2 * a.in + a.out;
    for (int idx = threadIdx.x; idx < a.in; idx += blockDim.x) {
        const int b = idx / M1, j = idx % M1;
        double v;
        if (j < a.nm) {
            double q0 = 0.0, qb = 0.0;
            const double* p0 = a.qpart + (size_t)a.slot[0] * PCH * a.nm + j;
            const double* pb = a.qpart + (size_t)a.slot[b] * PCH * a.nm + j;
            for (int c = 0; c < PCH; ++c) {
                q0 += p0[(size_t)c * a.nm];
                qb += pb[(size_t)c * a.nm];
            }
            v = (b == 0) ? q0 : qb - q0;
        } else {
            v = (b == 0) ? a.L[0] : a.L[b] - a.L[0];
        }
        x[idx] = (float)((v - in_mu[idx]) / in_sd[idx]);
    }
    __syncthreads();
    dense_warp_layer<true>(a.h1, a.in, a.W1, a.b1, x, y1);
    __syncthreads();
    dense_warp_layer<true>(a.h2, a.h1, a.W2, a.b2, y1, y2);
    __syncthreads();
    float* y3 = x;   // the features are no longer needed (in >= out)
    dense_warp_layer<false>(a.out, a.h2, a.W3, a.b3, y2, y3);
    __syncthreads();
    for (int j = threadIdx.x; j < a.out; j += blockDim.x) a.corr[j] = (double)y3[j] * out_sd[j] + out_mu[j];
}

// Ug = 4 h0 - 6 h1 + 4 h2 - h3 + Phi dq (nm = 0: the plain cubic extrapolation)
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
    const int nin = 4 * (nm + 1), nout = nm + 1;
    std::vector<double> st((size_t)2 * nin + 2 * nout);
    for (int i = 0; i < nin; ++i) {
        st[i] = imu ? imu[i] : 0.0;
        st[nin + i] = isd ? isd[i] : 1.0;
    }
    for (int i = 0; i < nout; ++i) {
        st[2 * nin + i] = omu ? omu[i] : 0.0;
        st[2 * nin + nout + i] = osd ? osd[i] : 1.0;
    }
    stats.upload(st, P.stream);
    hist.alloc((size_t)4 * n);
    qpart.alloc((size_t)4 * PCH * std::max(nm, 1));
    corr.alloc(nout);
    KL_CUDA(cudaMallocHost(&corrL_host, sizeof(double)));
    // the network's parameters are written on its own stream (training, set_params)
    if (net) KL_CUDA(cudaStreamSynchronize(net->stream));
    KL_CUDA(cudaStreamSynchronize(P.stream));
}

LearnedPredictor::~LearnedPredictor() {
    if (corrL_host) cudaFreeHost(corrL_host);
}

void LearnedPredictor::push(const double* dU, double L) {
    const int n = P.nfree;
    double* h = hist.get() + (size_t)head * n;
    KL_CUDA(cudaMemcpyAsync(h, dU, sizeof(double) * n, cudaMemcpyDeviceToDevice, P.stream));
    if (nm > 0) {
        project_kernel<<<dim3(PCH, nm), 256, 0, P.stream>>>(n, nm, Phi.get(), h, qpart.get() + (size_t)head * PCH * nm);
        count_launch();
        KL_CHECK_LAUNCH();
    }
    histL[head] = L;
    head = (head + 1) & 3;
    count = std::min(count + 1, 4);
}

bool LearnedPredictor::guess(double* dUg, double* Lg) {
    if (count < 4) return false;
    const int n = P.nfree;
    const int s[4] = {slot(0), slot(1), slot(2), slot(3)};
    const double Ls[4] = {histL[s[0]], histL[s[1]], histL[s[2]], histL[s[3]]};
    if (net) {
        InferArgs a;
        a.qpart = qpart.get();
        for (int b = 0; b < 4; ++b) {
            a.slot[b] = s[b];
            a.L[b] = Ls[b];
        }
        a.nm = nm;
        a.in = net->in;
        a.h1 = net->h1;
        a.h2 = net->h2;
        a.out = net->out;
        a.stats = stats.get();
        const float* W = net->params.get();
        a.W1 = W + net->oW1();
        a.b1 = W + net->ob1();
        a.W2 = W + net->oW2();
        a.b2 = W + net->ob2();
        a.W3 = W + net->oW3();
        a.b3 = W + net->ob3();
        a.corr = corr.get();
        const size_t smem = sizeof(float) * ((size_t)a.in + a.h1 + a.h2);
        infer_kernel<<<1, 1024, smem, P.stream>>>(a);
        count_launch();
        KL_CHECK_LAUNCH();
    }
    const int nq = net ? nm : 0;
    const double* H = hist.get();
    guess_kernel<<<ceil_div(n, 256), 256, sizeof(double) * std::max(nq, 1), P.stream>>>(
        n, nq, H + (size_t)s[0] * n, H + (size_t)s[1] * n, H + (size_t)s[2] * n, H + (size_t)s[3] * n, Phi.get(),
        corr.get(), dUg);
    count_launch();
    KL_CHECK_LAUNCH();
    double cL = 0.0;
    if (net) {
        KL_CUDA(cudaMemcpyAsync(corrL_host, corr.get() + nm, sizeof(double), cudaMemcpyDeviceToHost, P.stream));
        KL_CUDA(cudaStreamSynchronize(P.stream));
        cL = *corrL_host;
    }
    *Lg = 4.0 * Ls[0] - 6.0 * Ls[1] + 4.0 * Ls[2] - Ls[3] + cL;
    return true;
}

}  // namespace klsa
