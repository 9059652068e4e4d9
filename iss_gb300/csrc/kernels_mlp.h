// Launch wrappers of the proposal-network kernels (kernels_mlp.cu) and of the
// learned sampler's per-pair kernels (kernels_learned.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace iss {

// C[128][N] = A[128][K] * B[N][K]^T, bf16 row-major inputs, FP32 output;
// N in {32, 64, ..., 256}, K a multiple of 16 up to 256
cudaError_t launch_mma_selftest(const void* A, const void* B, int N, int K, float* C, int* err,
                                cudaStream_t s);

// bf16 weight images (mlp.h) from the FP32 parameters
cudaError_t launch_mlp_images(const float* params, void* img, cudaStream_t s);
// FP32 features [n][18] -> bf16 network input [n][32]
cudaError_t launch_features_to_bf16(const float* f, int64_t n, void* x, cudaStream_t s);
// out[n][64] = network(X); acts (optional, [4][n][128] bf16) keeps the hidden
// activations for the backward pass; with `records` the outputs are not
// written: the epilogue turns each row into its mixture record (64 floats,
// learned_record.cuh) instead
cudaError_t launch_mlp_forward(const void* img, const float* params, const void* X, int64_t n,
                               float* out, void* acts, int* err, int num_sms, cudaStream_t s,
                               float* records = nullptr);
// mean mixture negative log-likelihood of targets (K, nx, ny, nz): dout[n][64]
// = d(mean loss)/d(out); loss_base[step ? *step : 0] += sum of the row losses
cudaError_t launch_mlp_loss(const float* out, const void* target, int64_t n, float* dout,
                            double* loss_base, const int* step, cudaStream_t s);
// grad += d(mean loss)/d(params), from X, the activations and dout
cudaError_t launch_mlp_backward(const void* img, const void* X, const void* acts, const float* dout,
                                int64_t n, float* grad, int* err, int num_sms, cudaStream_t s);
// one Adam step (step count read from *step, which step_advance increments);
// clears grad and refreshes the images
cudaError_t launch_mlp_adam(float* params, float* m1, float* m2, float* grad, void* img,
                            const int* step, float lr, float b1, float b2, float eps,
                            cudaStream_t s);
cudaError_t launch_step_advance(int* step, cudaStream_t s);
// training batch of `batch` rows drawn with replacement from the data set
cudaError_t launch_gather_batch(const void* data_x, const void* data_t, int64_t n_data,
                                const int* step, uint32_t key0, uint32_t key1, int64_t batch,
                                void* x, void* tg, cudaStream_t s);

}  // namespace iss
