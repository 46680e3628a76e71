// mlp.cu -- small fully connected network (in -> h1 -> h2 -> out, GELU) with hand-written FP32
// forward, backward and Adam kernels.  Used by the learned arc-length predictor: trained on the
// GPU from equilibrium paths that the arc-length method generates, evaluated once per step.
//
// Layout: parameters in one contiguous FP32 buffer [W1 (h1 x in), b1, W2 (h2 x h1), b2,
// W3 (out x h2), b3], row-major weights; activations row-major (batch x features).
// Loss: L = 1/(2 B out) sum (Y - T)^2.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "mlp.h"

namespace klsa {

namespace {

constexpr int TILE = 16;

// C[M x N] = op(A) op(B) (+ bias[N]) ; op(A) is M x K: A row-major (M x K) or transposed
// (stored K x M); op(B) is K x N: B row-major (K x N) or transposed (stored N x K).
// epilogue: 0 plain, 1 add bias, 2 add bias and keep the pre-activation in Z, apply GELU.
// accumulate: C += result.
__global__ void gemm_kernel(int M, int N, int K, const float* __restrict__ A, bool ta, const float* __restrict__ B,
                            bool tb, const float* __restrict__ bias, float* __restrict__ C, float* __restrict__ Z,
                            int epilogue, bool accumulate) {
    __shared__ float As[TILE][TILE + 1], Bs[TILE][TILE + 1];
    int row = blockIdx.y * TILE + threadIdx.y, col = blockIdx.x * TILE + threadIdx.x;
    float acc = 0.f;
    for (int k0 = 0; k0 < K; k0 += TILE) {
        int ka = k0 + threadIdx.x, kb = k0 + threadIdx.y;
        int ar = blockIdx.y * TILE + threadIdx.y;
        As[threadIdx.y][threadIdx.x] = (ar < M && ka < K) ? (ta ? A[(size_t)ka * M + ar] : A[(size_t)ar * K + ka]) : 0.f;
        int bc = blockIdx.x * TILE + threadIdx.x;
        Bs[threadIdx.y][threadIdx.x] = (kb < K && bc < N) ? (tb ? B[(size_t)bc * K + kb] : B[(size_t)kb * N + bc]) : 0.f;
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TILE; ++kk) acc += As[threadIdx.y][kk] * Bs[kk][threadIdx.x];
        __syncthreads();
    }
    if (row >= M || col >= N) return;
    size_t o = (size_t)row * N + col;
    if (epilogue >= 1) acc += bias[col];
    if (epilogue == 2) {
        Z[o] = acc;
        acc = 0.5f * acc * (1.f + erff(acc * 0.70710678118654752f));
    }
    C[o] = accumulate ? C[o] + acc : acc;
}

// dZ = dH * gelu'(Z)
__global__ void gelu_back_kernel(int n, const float* __restrict__ Z, const float* __restrict__ dH, float* __restrict__ dZ) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float z = Z[i];
    float cdf = 0.5f * (1.f + erff(z * 0.70710678118654752f));
    float pdf = 0.3989422804014327f * expf(-0.5f * z * z);
    dZ[i] = dH[i] * (cdf + z * pdf);
}

// dY = (Y - T) / (B out), loss partial sums
__global__ void mse_grad_kernel(int n, float scale, const float* __restrict__ Y, const float* __restrict__ T,
                                float* __restrict__ dY, float* __restrict__ loss) {
    __shared__ float red[256];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float e = 0.f;
    if (i < n) {
        float d = Y[i] - T[i];
        dY[i] = d * scale;
        e = 0.5f * d * d * scale;
    }
    red[threadIdx.x] = e;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

// db[j] = sum_b dZ[b, j]
__global__ void colsum_kernel(int B, int N, const float* __restrict__ dZ, float* __restrict__ db) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    float s = 0.f;
    for (int b = 0; b < B; ++b) s += dZ[(size_t)b * N + j];
    db[j] = s;
}

__global__ void adam_kernel(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float gi = g[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void gather_rows_kernel(int B, int F, const int* __restrict__ idx, const float* __restrict__ src,
                                   float* __restrict__ dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * F) return;
    int b = i / F, f = i - b * F;
    dst[i] = src[(size_t)idx[b] * F + f];
}

void gemm(cudaStream_t s, int M, int N, int K, const float* A, bool ta, const float* B, bool tb, const float* bias,
          float* C, float* Z, int epi, bool acc) {
    dim3 block(TILE, TILE), grid(ceil_div(N, TILE), ceil_div(M, TILE));
    gemm_kernel<<<grid, block, 0, s>>>(M, N, K, A, ta, B, tb, bias, C, Z, epi, acc);
    count_launch();
}

}  // namespace

MLP::MLP(int nin, int nh1, int nh2, int nout, uint64_t seed) : in(nin), h1(nh1), h2(nh2), out(nout) {
    KL_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    nparams = (int64_t)h1 * in + h1 + (int64_t)h2 * h1 + h2 + (int64_t)out * h2 + out;
    std::vector<float> p(nparams, 0.f);
    std::mt19937_64 g(seed);
    auto init = [&](int64_t off, int fan_in, int fan_out, int64_t count) {
        float a = std::sqrt(6.f / (fan_in + fan_out));   // Glorot uniform
        std::uniform_real_distribution<float> U(-a, a);
        for (int64_t i = 0; i < count; ++i) p[off + i] = U(g);
    };
    init(oW1(), in, h1, (int64_t)h1 * in);
    init(oW2(), h1, h2, (int64_t)h2 * h1);
    init(oW3(), h2, out, (int64_t)out * h2);
    params.upload(p, stream);
    grad.alloc(nparams);
    m.alloc(nparams);
    v.alloc(nparams);
    m.zero(stream);
    v.zero(stream);
    loss.alloc(1);
    KL_CUDA(cudaStreamSynchronize(stream));
}

MLP::~MLP() {
    if (stream) cudaStreamDestroy(stream);
}

void MLP::ensure_batch(int B) {
    if (B <= cap) return;
    cap = B;
    Z1.alloc((size_t)B * h1); H1.alloc((size_t)B * h1);
    Z2.alloc((size_t)B * h2); H2.alloc((size_t)B * h2);
    Y.alloc((size_t)B * out); dY.alloc((size_t)B * out);
    dH2.alloc((size_t)B * h2); dZ2.alloc((size_t)B * h2);
    dH1.alloc((size_t)B * h1); dZ1.alloc((size_t)B * h1);
    Xb.alloc((size_t)B * in); Tb.alloc((size_t)B * out);
    idx.alloc(B);
}

void MLP::forward(const float* dX, int B) {
    ensure_batch(B);
    const float* P = params.get();
    gemm(stream, B, h1, in, dX, false, P + oW1(), true, P + ob1(), H1.get(), Z1.get(), 2, false);
    gemm(stream, B, h2, h1, H1.get(), false, P + oW2(), true, P + ob2(), H2.get(), Z2.get(), 2, false);
    gemm(stream, B, out, h2, H2.get(), false, P + oW3(), true, P + ob3(), Y.get(), nullptr, 1, false);
    KL_CHECK_LAUNCH();
}

float MLP::loss_grad(const float* dX, const float* dT, int B) {
    forward(dX, B);
    const float* P = params.get();
    float* G = grad.get();
    KL_CUDA(cudaMemsetAsync(loss.get(), 0, sizeof(float), stream));
    int n = B * out;
    mse_grad_kernel<<<ceil_div(n, 256), 256, 0, stream>>>(n, 1.f / (float)n, Y.get(), dT, dY.get(), loss.get());
    count_launch();
    // layer 3
    gemm(stream, out, h2, B, dY.get(), true, H2.get(), false, nullptr, G + oW3(), nullptr, 0, false);
    colsum_kernel<<<ceil_div(out, 128), 128, 0, stream>>>(B, out, dY.get(), G + ob3());
    count_launch();
    gemm(stream, B, h2, out, dY.get(), false, P + oW3(), false, nullptr, dH2.get(), nullptr, 0, false);
    gelu_back_kernel<<<ceil_div((int64_t)B * h2, 256), 256, 0, stream>>>(B * h2, Z2.get(), dH2.get(), dZ2.get());
    count_launch();
    // layer 2
    gemm(stream, h2, h1, B, dZ2.get(), true, H1.get(), false, nullptr, G + oW2(), nullptr, 0, false);
    colsum_kernel<<<ceil_div(h2, 128), 128, 0, stream>>>(B, h2, dZ2.get(), G + ob2());
    count_launch();
    gemm(stream, B, h1, h2, dZ2.get(), false, P + oW2(), false, nullptr, dH1.get(), nullptr, 0, false);
    gelu_back_kernel<<<ceil_div((int64_t)B * h1, 256), 256, 0, stream>>>(B * h1, Z1.get(), dH1.get(), dZ1.get());
    count_launch();
    // layer 1
    gemm(stream, h1, in, B, dZ1.get(), true, dX, false, nullptr, G + oW1(), nullptr, 0, false);
    colsum_kernel<<<ceil_div(h1, 128), 128, 0, stream>>>(B, h1, dZ1.get(), G + ob1());
    count_launch();
    KL_CHECK_LAUNCH();
    float l = 0.f;
    KL_CUDA(cudaMemcpyAsync(&l, loss.get(), sizeof(float), cudaMemcpyDeviceToHost, stream));
    KL_CUDA(cudaStreamSynchronize(stream));
    return l;
}

void MLP::adam_step(float lr) {
    ++t_adam;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float c1 = 1.f - std::pow(b1, (float)t_adam), c2 = 1.f - std::pow(b2, (float)t_adam);
    adam_kernel<<<ceil_div(nparams, 256), 256, 0, stream>>>((int)nparams, params.get(), grad.get(), m.get(), v.get(), lr,
                                                             b1, b2, eps, c1, c2);
    count_launch();
}

float MLP::train(const float* hX, const float* hT, int nsamples, int epochs, int B, float lr, uint64_t seed) {
    DevBuf<float> X, T;
    X.upload(hX, (size_t)nsamples * in, stream);
    T.upload(hT, (size_t)nsamples * out, stream);
    B = std::min(B, nsamples);
    ensure_batch(B);
    std::mt19937_64 g(seed);
    std::vector<int> perm(nsamples);
    for (int i = 0; i < nsamples; ++i) perm[i] = i;
    float last = 0.f;
    int nb = nsamples / B;
    for (int ep = 0; ep < epochs; ++ep) {
        std::shuffle(perm.begin(), perm.end(), g);
        float lr_ep = lr * 0.5f * (1.f + std::cos(3.14159265f * ep / std::max(1, epochs)));   // cosine schedule
        double acc = 0.0;
        for (int b = 0; b < nb; ++b) {
            idx.upload(perm.data() + (size_t)b * B, B, stream);
            gather_rows_kernel<<<ceil_div((int64_t)B * in, 256), 256, 0, stream>>>(B, in, idx.get(), X.get(), Xb.get());
            gather_rows_kernel<<<ceil_div((int64_t)B * out, 256), 256, 0, stream>>>(B, out, idx.get(), T.get(), Tb.get());
            count_launch(2);
            acc += loss_grad(Xb.get(), Tb.get(), B);
            adam_step(lr_ep);
        }
        last = (float)(acc / std::max(nb, 1));
    }
    KL_CUDA(cudaStreamSynchronize(stream));
    return last;
}

}  // namespace klsa
