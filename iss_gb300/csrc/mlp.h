// The conditional proposal network of the learned sampler: sizes, the flat
// parameter layout and the bf16 weight images the tensor-core kernels read.
//
// Network: 18 conditioning features (padded to 32) -> 4 hidden layers of 128
// (ReLU) -> 64 outputs, of which 48 parameterise an 8-component mixture over
// the local-rest-frame momentum in (K, n), K = (E - m) / T, n = p / |p|:
//   out[0..7]    mixture logits
//   out[8..15]   mu_k, location of ln K (log-normal in K)
//   out[16..23]  s_k = ln sigma_k (clamped to [kLogSigMin, kLogSigMax])
//   out[24..47]  v_k (3 per component): von Mises-Fisher direction v / |v|,
//                concentration |v|
// Parameters are FP32 masters in one flat array, row-major W[out][in] then
// b[out] per layer; the kernels read bf16 copies laid out as the canonical
// K-major shared-memory tiles of tc05.cuh (forward: W[out][in]; backward:
// W^T[in][out]), so a tile is loaded by a linear copy.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace iss {
namespace mlp {

constexpr int kFeatures = 18;
constexpr int kIn0 = 32;      // K of the first layer (features zero-padded)
constexpr int kHid = 128;
constexpr int kOut = 64;      // output layer rows (48 used)
constexpr int kOutUsed = 48;
constexpr int kComp = 8;
constexpr int kLayers = 5;
constexpr int kTile = 128;    // rows (samples) per CTA tile
constexpr float kLogSigMin = -4.0f, kLogSigMax = 1.5f;

__host__ __device__ constexpr int dim_in(int l) { return l == 0 ? kIn0 : kHid; }
__host__ __device__ constexpr int dim_out(int l) { return l == kLayers - 1 ? kOut : kHid; }

// flat FP32 parameter array: W0 b0 W1 b1 ... W4 b4
__host__ __device__ constexpr int64_t w_offset(int l) {
    int64_t o = 0;
    for (int i = 0; i < l; i++) o += static_cast<int64_t>(dim_out(i)) * dim_in(i) + dim_out(i);
    return o;
}
__host__ __device__ constexpr int64_t b_offset(int l) {
    return w_offset(l) + static_cast<int64_t>(dim_out(l)) * dim_in(l);
}
constexpr int64_t kNumParams = w_offset(kLayers);

// bf16 images (element offsets): forward images of all layers back to back,
// then the backward (transposed) images of layers 1..4
__host__ __device__ constexpr int64_t fwd_img_offset(int l) {
    int64_t o = 0;
    for (int i = 0; i < l; i++) o += static_cast<int64_t>(dim_out(i)) * dim_in(i);
    return o;
}
constexpr int64_t kFwdImgElems = fwd_img_offset(kLayers);
__host__ __device__ constexpr int64_t bwd_img_offset(int l) {   // l >= 1
    int64_t o = kFwdImgElems;
    for (int i = 1; i < l; i++) o += static_cast<int64_t>(dim_out(i)) * dim_in(i);
    return o;
}
constexpr int64_t kImgElems = bwd_img_offset(kLayers);

static_assert(kNumParams == 62016, "parameter count");
static_assert(kFwdImgElems * 2 == 122880, "forward image bytes");

}  // namespace mlp
}  // namespace iss
