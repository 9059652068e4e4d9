// Host side of the learned proposal: the network's device state (FP32
// masters, Adam moments, bf16 images), its training loop on momenta drawn by
// the plain sampler, and the per-(species, cell) mixture tables the learned
// sampler reads.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "devbuf.h"
#include "mlp.h"

namespace iss {

struct Learned {
    // network
    DevBuf<float> params, m1, m2, grad;
    DevBuf<uint16_t> img;       // bf16 images (mlp.h)
    DevBuf<int> step, err;
    DevBuf<double> loss;
    bool have_weights = false;
    // scratch of forward / loss / backward
    DevBuf<uint16_t> x, acts;
    DevBuf<float> feat, out, dout;
    DevBuf<float4> tg;
    // training set: bf16 features [n][32] and targets (K, n) [n]
    DevBuf<uint16_t> data_x;
    DevBuf<float4> data_t;
    int64_t n_data = 0;
    std::string error;

    void release_all();
    // FP32 parameters from the host (kNumParams floats); images rebuilt
    cudaError_t set_params(const float* host, cudaStream_t s);
    cudaError_t get_params(float* host, cudaStream_t s);
    // deterministic initial parameters (uniform fan-in scaling, output layer
    // biased to a broad mixture)
    static void initial_params(uint64_t seed, std::vector<float>* out);
    // forward pass of n feature rows (FP32 [n][18], host) -> out [n][64] (host)
    cudaError_t forward_host(const float* feat, int64_t n, float* out, int num_sms, cudaStream_t s);
    // mean loss and its parameter gradient for n rows (host in / out)
    cudaError_t loss_grad_host(const float* feat, const float* targets, int64_t n, double* loss,
                               float* grad_out, int num_sms, cudaStream_t s);
    // n_steps Adam steps on batches drawn from the training set; loss per step
    // to loss_curve (if not null)
    cudaError_t train(int n_steps, int64_t batch, float lr, uint32_t key0, uint32_t key1,
                      double* loss_curve, int num_sms, cudaStream_t s);
    // device error flag of the last network kernels (bounded waits that gave up)
    int device_error(cudaStream_t s);
};

}  // namespace iss
