// Mixture record of one (species, cell) pair from the network's outputs
// (layout of kPairFloats in device_common.cuh): per component k the
// cumulative weight, log-normaliser c_k = ln w_k - ln sigma_k - ln sqrt(2 pi)
// + ln(kappa / (4 pi sinh kappa)), mu_k, sigma_k, v_k and kappa_k = |v_k|.
#pragma once

#include <cuda_runtime.h>

namespace iss {

__device__ __forceinline__ float log_vmf_norm_f(float kappa) {
    const float l4pi = 2.5310242469692907f;   // ln(4 pi)
    if (kappa < 1e-3f) return -l4pi - kappa * kappa * (1.0f / 6.0f);
    return -l4pi - kappa + logf(2.0f * kappa) - logf(-expm1f(-2.0f * kappa));
}

// z: the 48 used outputs of the row; r: 64 floats
__device__ __forceinline__ void mixture_record(const float* z, float* r) {
    float lmax = -INFINITY;
#pragma unroll
    for (int k = 0; k < 8; k++) lmax = fmaxf(lmax, z[k]);
    float se = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) se += expf(z[k] - lmax);
    const float lse = lmax + logf(se);
    float cw = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        cw += expf(z[k] - lse);
        const float sg = fminf(fmaxf(z[16 + k], -4.0f), 1.5f);
        const float vx = z[24 + 3 * k], vy = z[25 + 3 * k], vz = z[26 + 3 * k];
        const float kap = sqrtf(vx * vx + vy * vy + vz * vz);
        r[8 * k + 0] = k < 7 ? cw : 1.0f;
        r[8 * k + 1] = z[k] - lse - sg - 0.91893853320467274f + log_vmf_norm_f(kap);
        r[8 * k + 2] = z[8 + k];
        r[8 * k + 3] = expf(sg);
        r[8 * k + 4] = vx;
        r[8 * k + 5] = vy;
        r[8 * k + 6] = vz;
        r[8 * k + 7] = kap;
    }
}

}  // namespace iss
