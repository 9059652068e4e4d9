// Host side of the learned proposal network (learned.h).
#include "learned.h"

#include <cmath>
#include <cstring>

#include "kernels_mlp.h"

namespace iss {

using namespace mlp;

#define LTRY(call)                              \
    do {                                        \
        cudaError_t _e = (call);                \
        if (_e != cudaSuccess) return _e;       \
    } while (0)

void Learned::release_all() {
    params.release();
    m1.release();
    m2.release();
    grad.release();
    img.release();
    step.release();
    err.release();
    loss.release();
    x.release();
    acts.release();
    feat.release();
    out.release();
    dout.release();
    tg.release();
    data_x.release();
    data_t.release();
    n_data = 0;
    have_weights = false;
}

namespace {

uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double uniform01(uint64_t& s) { return static_cast<double>(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

cudaError_t ensure_network(Learned& L) {
    LTRY(L.params.reserve(kNumParams));
    LTRY(L.m1.reserve(kNumParams));
    LTRY(L.m2.reserve(kNumParams));
    LTRY(L.grad.reserve(kNumParams));
    LTRY(L.img.reserve(kImgElems));
    LTRY(L.step.reserve(1));
    LTRY(L.err.reserve(1));
    return cudaSuccess;
}

}  // namespace

void Learned::initial_params(uint64_t seed, std::vector<float>* out) {
    std::vector<float>& p = *out;
    p.assign(kNumParams, 0.0f);
    uint64_t s = seed ^ 0x5EEDF00Dull;
    for (int l = 0; l < kLayers; l++) {
        const int K = dim_in(l), N = dim_out(l);
        const int fan_in = (l == 0) ? kFeatures : K;
        const double a = (l == kLayers - 1) ? 0.1 * std::sqrt(3.0 / fan_in) : std::sqrt(6.0 / fan_in);
        float* W = p.data() + w_offset(l);
        for (int o = 0; o < N; o++)
            for (int i = 0; i < K; i++) {
                const bool pad = (l == 0 && i >= kFeatures) || (l == kLayers - 1 && o >= kOutUsed);
                const double u = uniform01(s);
                W[o * K + i] = pad ? 0.0f : static_cast<float>((2.0 * u - 1.0) * a);
            }
    }
    // output biases: equal weights, log-normal locations spread over
    // K = 0.25 .. 6.7, sigma = 0.5, small random direction vectors
    float* b = p.data() + b_offset(kLayers - 1);
    for (int k = 0; k < kComp; k++) {
        b[k] = 0.0f;
        b[8 + k] = static_cast<float>(std::log(0.25 * std::pow(1.6, k)));
        b[16 + k] = static_cast<float>(std::log(0.5));
        for (int j = 0; j < 3; j++) b[24 + 3 * k + j] = static_cast<float>(0.2 * (uniform01(s) - 0.5));
    }
}

cudaError_t Learned::set_params(const float* host, cudaStream_t s) {
    LTRY(ensure_network(*this));
    LTRY(cudaMemcpyAsync(params.ptr, host, sizeof(float) * kNumParams, cudaMemcpyHostToDevice, s));
    LTRY(cudaMemsetAsync(m1.ptr, 0, sizeof(float) * kNumParams, s));
    LTRY(cudaMemsetAsync(m2.ptr, 0, sizeof(float) * kNumParams, s));
    LTRY(cudaMemsetAsync(grad.ptr, 0, sizeof(float) * kNumParams, s));
    LTRY(cudaMemsetAsync(img.ptr, 0, sizeof(uint16_t) * kImgElems, s));
    LTRY(cudaMemsetAsync(step.ptr, 0, sizeof(int), s));
    LTRY(cudaMemsetAsync(err.ptr, 0, sizeof(int), s));
    LTRY(launch_mlp_images(params.ptr, img.ptr, s));
    LTRY(cudaStreamSynchronize(s));
    have_weights = true;
    return cudaSuccess;
}

cudaError_t Learned::get_params(float* host, cudaStream_t s) {
    LTRY(cudaMemcpyAsync(host, params.ptr, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost, s));
    return cudaStreamSynchronize(s);
}

int Learned::device_error(cudaStream_t s) {
    int e = 0;
    if (!err.ptr) return 0;
    if (cudaMemcpyAsync(&e, err.ptr, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    return e;
}

cudaError_t Learned::forward_host(const float* f, int64_t n, float* o, int num_sms, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    LTRY(feat.reserve(static_cast<size_t>(n) * kFeatures));
    LTRY(x.reserve(static_cast<size_t>(n) * kIn0));
    LTRY(out.reserve(static_cast<size_t>(n) * kOut));
    LTRY(cudaMemcpyAsync(feat.ptr, f, sizeof(float) * kFeatures * n, cudaMemcpyHostToDevice, s));
    LTRY(launch_features_to_bf16(feat.ptr, n, x.ptr, s));
    LTRY(launch_mlp_forward(img.ptr, params.ptr, x.ptr, n, out.ptr, nullptr, err.ptr, num_sms, s));
    LTRY(cudaMemcpyAsync(o, out.ptr, sizeof(float) * kOut * n, cudaMemcpyDeviceToHost, s));
    return cudaStreamSynchronize(s);
}

cudaError_t Learned::loss_grad_host(const float* f, const float* targets, int64_t n, double* loss_out,
                                    float* grad_out, int num_sms, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    LTRY(feat.reserve(static_cast<size_t>(n) * kFeatures));
    LTRY(x.reserve(static_cast<size_t>(n) * kIn0));
    LTRY(out.reserve(static_cast<size_t>(n) * kOut));
    LTRY(dout.reserve(static_cast<size_t>(n) * kOut));
    LTRY(acts.reserve(static_cast<size_t>(n) * kHid * (kLayers - 1)));
    LTRY(tg.reserve(static_cast<size_t>(n)));
    LTRY(loss.reserve(1));
    LTRY(cudaMemcpyAsync(feat.ptr, f, sizeof(float) * kFeatures * n, cudaMemcpyHostToDevice, s));
    LTRY(cudaMemcpyAsync(tg.ptr, targets, sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    LTRY(cudaMemsetAsync(loss.ptr, 0, sizeof(double), s));
    LTRY(cudaMemsetAsync(grad.ptr, 0, sizeof(float) * kNumParams, s));
    LTRY(launch_features_to_bf16(feat.ptr, n, x.ptr, s));
    LTRY(launch_mlp_forward(img.ptr, params.ptr, x.ptr, n, out.ptr, acts.ptr, err.ptr, num_sms, s));
    LTRY(launch_mlp_loss(out.ptr, tg.ptr, n, dout.ptr, loss.ptr, nullptr, s));
    LTRY(launch_mlp_backward(img.ptr, x.ptr, acts.ptr, dout.ptr, n, grad.ptr, err.ptr, num_sms, s));
    double lsum = 0.0;
    LTRY(cudaMemcpyAsync(&lsum, loss.ptr, sizeof(double), cudaMemcpyDeviceToHost, s));
    LTRY(cudaMemcpyAsync(grad_out, grad.ptr, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost, s));
    LTRY(cudaMemsetAsync(grad.ptr, 0, sizeof(float) * kNumParams, s));
    LTRY(cudaStreamSynchronize(s));
    *loss_out = lsum / static_cast<double>(n);
    return cudaSuccess;
}

cudaError_t Learned::train(int n_steps, int64_t batch, float lr, uint32_t key0, uint32_t key1,
                           double* loss_curve, int num_sms, cudaStream_t s) {
    if (n_steps <= 0 || n_data <= 0) return cudaSuccess;
    LTRY(x.reserve(static_cast<size_t>(batch) * kIn0));
    LTRY(out.reserve(static_cast<size_t>(batch) * kOut));
    LTRY(dout.reserve(static_cast<size_t>(batch) * kOut));
    LTRY(acts.reserve(static_cast<size_t>(batch) * kHid * (kLayers - 1)));
    LTRY(tg.reserve(static_cast<size_t>(batch)));
    LTRY(loss.reserve(static_cast<size_t>(n_steps)));
    LTRY(cudaMemsetAsync(loss.ptr, 0, sizeof(double) * n_steps, s));
    LTRY(cudaMemsetAsync(step.ptr, 0, sizeof(int), s));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    auto one_step = [&]() -> cudaError_t {
        LTRY(launch_gather_batch(data_x.ptr, data_t.ptr, n_data, step.ptr, key0, key1, batch, x.ptr,
                                 tg.ptr, s));
        LTRY(launch_mlp_forward(img.ptr, params.ptr, x.ptr, batch, out.ptr, acts.ptr, err.ptr,
                                num_sms, s));
        LTRY(launch_mlp_loss(out.ptr, tg.ptr, batch, dout.ptr, loss.ptr, step.ptr, s));
        LTRY(launch_mlp_backward(img.ptr, x.ptr, acts.ptr, dout.ptr, batch, grad.ptr, err.ptr,
                                 num_sms, s));
        LTRY(launch_mlp_adam(params.ptr, m1.ptr, m2.ptr, grad.ptr, img.ptr, step.ptr, lr, b1, b2, eps,
                             s));
        LTRY(launch_step_advance(step.ptr, s));
        return cudaSuccess;
    };
    // the first step runs eagerly (one-time kernel attributes), the others
    // replay one captured graph of the step
    LTRY(one_step());
    if (n_steps > 1) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        LTRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const cudaError_t ce = one_step();
        const cudaError_t ee = cudaStreamEndCapture(s, &graph);
        if (ce != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return ce;
        }
        LTRY(ee);
        cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        LTRY(e);
        for (int i = 1; i < n_steps && e == cudaSuccess; i++) e = cudaGraphLaunch(exec, s);
        const cudaError_t se = cudaStreamSynchronize(s);
        cudaGraphExecDestroy(exec);
        LTRY(e);
        LTRY(se);
    }
    if (loss_curve) {
        LTRY(cudaMemcpyAsync(loss_curve, loss.ptr, sizeof(double) * n_steps, cudaMemcpyDeviceToHost, s));
        LTRY(cudaStreamSynchronize(s));
        for (int i = 0; i < n_steps; i++) loss_curve[i] /= static_cast<double>(batch);
    }
    return cudaStreamSynchronize(s);
}

}  // namespace iss
