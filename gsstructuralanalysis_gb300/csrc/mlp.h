// mlp.h -- fully connected in -> h1 -> h2 -> out network with GELU, FP32, on the device.
#pragma once

#include <algorithm>
#include <cstdint>

#include "common.cuh"

namespace klsa {

struct MLP {
    int in, h1, h2, out;
    int64_t nparams = 0;
    cudaStream_t stream = nullptr;
    DevBuf<float> params, grad, m, v, loss;
    DevBuf<float> Z1, H1, Z2, H2, Y, dY, dH2, dZ2, dH1, dZ1, Xb, Tb;
    DevBuf<int> idx;
    int cap = 0;
    int t_adam = 0;

    MLP(int nin, int nh1, int nh2, int nout, uint64_t seed);
    ~MLP();
    int64_t oW1() const { return 0; }
    int64_t ob1() const { return (int64_t)h1 * in; }
    int64_t oW2() const { return ob1() + h1; }
    int64_t ob2() const { return oW2() + (int64_t)h2 * h1; }
    int64_t oW3() const { return ob2() + h2; }
    int64_t ob3() const { return oW3() + (int64_t)out * h2; }
    void ensure_batch(int B);
    // Y = net(X) for a device batch (B x in); result in this->Y
    void forward(const float* dX, int B);
    // forward + backward of the MSE loss; gradient in this->grad, returns the loss
    float loss_grad(const float* dX, const float* dT, int B);
    void adam_step(float lr);
    // mini-batch Adam with a cosine learning-rate schedule; returns the last epoch's mean loss
    float train(const float* hX, const float* hT, int nsamples, int epochs, int B, float lr, uint64_t seed);
};

}  // namespace klsa
