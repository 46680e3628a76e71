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

// qslot[c * nm + j] = sum over chunk c of Phi_j . u (fixed order within the chunk); the blocks
// of mode 0 also copy u into the history ring (copy)
__global__ void __launch_bounds__(256) project_kernel(int n, int nm, const double* __restrict__ Phi,
                                                      const double* __restrict__ u, double* __restrict__ qslot,
                                                      double* __restrict__ copy) {
    __shared__ double red[8];
    const int j = blockIdx.y, c = blockIdx.x;
    const int len = (n + PCH - 1) / PCH, lo = c * len, hi = min(n, lo + len);
    const double* ph = Phi + (size_t)j * n;
    double s = 0.0;
#pragma unroll 4
    for (int i = lo + threadIdx.x; i < hi; i += 256) {
        const double ui = u[i];
        s += ph[i] * ui;
        if (j == 0) copy[i] = ui;
    }
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
    float *y1, *y2;        // hidden activations (predictor's own scratch)
    double* corr;          // out: destandardised network output
};

constexpr int ROWS_PER_CTA = 8;   // one warp per output row

// one output row of a dense layer: the lanes walk the weight row in 128-byte pieces with four
// independent partial sums (four loads in flight per lane), then the warp adds them up
__device__ __forceinline__ float dense_row(const float* __restrict__ w, const float* x, int nin, int lane) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int k = lane;
    for (; k + 96 < nin; k += 128) {
        s0 = fmaf(x[k], w[k], s0);
        s1 = fmaf(x[k + 32], w[k + 32], s1);
        s2 = fmaf(x[k + 64], w[k + 64], s2);
        s3 = fmaf(x[k + 96], w[k + 96], s3);
    }
    for (; k < nin; k += 32) s0 = fmaf(x[k], w[k], s0);
    float acc = (s0 + s1) + (s2 + s3);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }

// features of the last four points (every CTA builds them in shared memory) and the first layer
__global__ void __launch_bounds__(256) infer_l1_kernel(InferArgs a) {
    extern __shared__ float x[];
    const int M1 = a.nm + 1;
    const double *in_mu = a.stats, *in_sd = a.stats + a.in;
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
    const int lane = threadIdx.x & 31, r = blockIdx.x * ROWS_PER_CTA + (threadIdx.x >> 5);
    if (r < a.h1) {
        const float acc = dense_row(a.W1 + (size_t)r * a.in, x, a.in, lane);
        if (lane == 0) a.y1[r] = gelu(acc + a.b1[r]);
    }
}

// a hidden or output layer: the input row staged in shared memory, one warp per output row
template <int LAYER>
__global__ void __launch_bounds__(256) infer_layer_kernel(InferArgs a) {
    extern __shared__ float x[];
    const int nin = LAYER == 2 ? a.h1 : a.h2, nout = LAYER == 2 ? a.h2 : a.out;
    const float* src = LAYER == 2 ? a.y1 : a.y2;
    for (int k = threadIdx.x; k < nin; k += blockDim.x) x[k] = src[k];
    __syncthreads();
    const int lane = threadIdx.x & 31, r = blockIdx.x * ROWS_PER_CTA + (threadIdx.x >> 5);
    if (r >= nout) return;
    const float* W = LAYER == 2 ? a.W2 : a.W3;
    const float acc = dense_row(W + (size_t)r * nin, x, nin, lane);
    if (lane == 0) {
        if (LAYER == 2) {
            a.y2[r] = gelu(acc + a.b2[r]);
        } else {
            const double *out_mu = a.stats + 2 * a.in, *out_sd = a.stats + 2 * a.in + a.out;
            a.corr[r] = (double)(acc + a.b3[r]) * out_sd[r] + out_mu[r];
        }
    }
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
    if (net) {
        hid.alloc((size_t)net->h1 + net->h2);
    }
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
    if (nm > 0) {
        project_kernel<<<dim3(PCH, nm), 256, 0, P.stream>>>(n, nm, Phi.get(), dU, qpart.get() + (size_t)head * PCH * nm, h);
        count_launch();
        KL_CHECK_LAUNCH();
    } else {
        KL_CUDA(cudaMemcpyAsync(h, dU, sizeof(double) * n, cudaMemcpyDeviceToDevice, P.stream));
    }
    histL[head] = L;
    head = (head + 1) & 3;
    count = std::min(count + 1, 4);
}

bool LearnedPredictor::guess(double* dUg, double* Lg) {
    if (!launch_guess(dUg, Lg)) return false;
    if (net) {
        KL_CUDA(cudaMemcpyAsync(corrL_host, corr.get() + nm, sizeof(double), cudaMemcpyDeviceToHost, P.stream));
        KL_CUDA(cudaStreamSynchronize(P.stream));
        *Lg += *corrL_host;
    }
    return true;
}

bool LearnedPredictor::guess_deferred(double* dUg, double* Lg, const double** Lcorr) {
    if (!launch_guess(dUg, Lg)) return false;
    *Lcorr = net ? corr.get() + nm : nullptr;
    return true;
}

// the network (if any) and the guess kernel; *Lcubic = the cubic extrapolation of the load factor
bool LearnedPredictor::launch_guess(double* dUg, double* Lcubic) {
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
        a.y1 = hid.get();
        a.y2 = hid.get() + a.h1;
        a.corr = corr.get();
        infer_l1_kernel<<<ceil_div(a.h1, ROWS_PER_CTA), 256, sizeof(float) * a.in, P.stream>>>(a);
        count_launch();
        infer_layer_kernel<2><<<ceil_div(a.h2, ROWS_PER_CTA), 256, sizeof(float) * a.h1, P.stream>>>(a);
        count_launch();
        infer_layer_kernel<3><<<ceil_div(a.out, ROWS_PER_CTA), 256, sizeof(float) * a.h2, P.stream>>>(a);
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
    *Lcubic = 4.0 * Ls[0] - 6.0 * Ls[1] + 4.0 * Ls[2] - Ls[3];
    return true;
}

}  // namespace klsa
