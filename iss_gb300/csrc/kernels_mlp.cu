// The conditional proposal network of the learned sampler on the tensor
// cores: forward (inference and training), mixture negative log-likelihood,
// backward, Adam, plus a single-tile GEMM self-test of the tcgen05 path.
//
// Every GEMM is a tcgen05.mma (kind::f16, bf16 operands from shared memory,
// FP32 accumulator in TMEM) issued by one thread of a 128-thread CTA; thread t
// owns row t of a 128-row tile, which is TMEM lane t, and runs that row's
// epilogue from tcgen05.ld.  Operands are written to shared memory by the
// threads themselves in the canonical K-major layout (tc05.cuh), transposed
// where a GEMM contracts over the tile's rows (the weight gradients).
#include <cuda_bf16.h>

#include "device_common.cuh"
#include "kernels_mlp.h"
#include "learned_record.cuh"
#include "mlp.h"
#include "tc05.cuh"

namespace iss {
namespace {

using namespace tc05;
using namespace mlp;

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ void sync_for_mma() {
    fence_smem_to_async();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
}

__device__ __forceinline__ void barrier_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// ---------------------------------------------------------------------------
// self-test: C[128][N] = A[128][K] * B[N][K]^T in one CTA

__global__ void __launch_bounds__(128, 1)
mma_selftest_kernel(const __nv_bfloat16* __restrict__ A, const __nv_bfloat16* __restrict__ B, int N,
                    int K, uint32_t ncols, float* __restrict__ C, int* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sA = smem;
    uint8_t* sB = smem + 128 * K * 2;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sB + N * K * 2);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    const int t = threadIdx.x, warp = t >> 5;
    for (int c = 0; c < K / 8; c++)
        *reinterpret_cast<uint4*>(sA + kmajor_offset(t, 8 * c, K)) =
            reinterpret_cast<const uint4*>(A + static_cast<size_t>(t) * K)[c];
    for (int r = t; r < N; r += 128)
        for (int c = 0; c < K / 8; c++)
            *reinterpret_cast<uint4*>(sB + kmajor_offset(r, 8 * c, K)) =
                reinterpret_cast<const uint4*>(B + static_cast<size_t>(r) * K)[c];
    if (t == 0) {
        mbar_init(bar, 1);
        barrier_init_fence();
    }
    if (warp == 0) {
        tmem_alloc(tslot, ncols);
        tmem_relinquish();
    }
    sync_for_mma();
    const uint32_t tmem = *tslot;
    if (t == 0) {
        const uint32_t id = idesc_bf16_f32(128, N);
        for (int ks = 0; ks < K / 16; ks++)
            mma_bf16(tmem, kslice_desc(smem_addr(sA), K, ks), kslice_desc(smem_addr(sB), K, ks), id,
                     ks > 0);
        mma_commit(bar);
    }
    const int ok = __syncthreads_and(mbar_wait(bar, 0, err, 1));
    fence_after_sync();
    if (ok) {
        for (int c0 = 0; c0 < N; c0 += 32) {
            float v[32];
            tmem_ld32(tmem_lane_addr(tmem, warp, c0), v);
#pragma unroll
            for (int j = 0; j < 32; j++) C[static_cast<size_t>(t) * N + c0 + j] = v[j];
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------
// forward: out = f(X) for n rows; hidden activations kept for training.
//
// kFwdWG warpgroups per CTA share the weight images in shared memory; each
// warpgroup g owns one 128-row tile at a time, its own activation buffer
// (which first holds the tile's inputs), TMEM columns [128 g, 128 g + 128),
// an mbarrier and a named barrier, so one tile's epilogue overlaps another
// tile's GEMMs on the tensor core.

constexpr int kFwdWG = 3;
constexpr int kFwdThreads = 128 * kFwdWG;
// biases of the hidden layers and the used outputs, staged in shared memory
constexpr int kFwdBias = (kLayers - 1) * kHid + kOut;
constexpr int kFwdSmem = static_cast<int>(kFwdImgElems * 2) + kFwdWG * kTile * kHid * 2 + 64 + kFwdBias * 4;

// barrier over the 128 threads of warpgroup `id - 1` (named barrier `id`)
__device__ __forceinline__ void wg_sync(int id) {
    asm volatile("bar.sync %0, 128;" :: "r"(id) : "memory");
}
__device__ __forceinline__ bool wg_sync_and(int id, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "barrier.red.and.pred q, %2, 128, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r) : "r"(static_cast<uint32_t>(v)), "r"(id) : "memory");
    return r != 0;
}
__device__ __forceinline__ void wg_sync_for_mma(int id) {
    fence_smem_to_async();
    fence_before_sync();
    wg_sync(id);
    fence_after_sync();
}

__global__ void __launch_bounds__(kFwdThreads, 1)
mlp_fwd_kernel(const __nv_bfloat16* __restrict__ img, const float* __restrict__ params,
               const __nv_bfloat16* __restrict__ X, int64_t n, float* __restrict__ out,
               __nv_bfloat16* __restrict__ acts, float* __restrict__ records,
               int* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sW = smem;
    const int g = threadIdx.x >> 7;            // warpgroup
    const int t = threadIdx.x & 127;           // row of the warpgroup's tile
    const int warp = threadIdx.x >> 5;
    const int bar_id = 1 + g;
    uint8_t* sH = sW + kFwdImgElems * 2 + g * (kTile * kHid * 2);   // inputs, then activations
    uint64_t* bars = reinterpret_cast<uint64_t*>(sW + kFwdImgElems * 2 + kFwdWG * kTile * kHid * 2);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + kFwdWG);
    float* sBias = reinterpret_cast<float*>(sW + kFwdImgElems * 2 + kFwdWG * kTile * kHid * 2 + 64);
    {
        const uint4* src = reinterpret_cast<const uint4*>(img);
        uint4* dst = reinterpret_cast<uint4*>(sW);
        for (int i = threadIdx.x; i < static_cast<int>(kFwdImgElems * 2 / 16); i += kFwdThreads)
            dst[i] = src[i];
        for (int i = threadIdx.x; i < kFwdBias; i += kFwdThreads) {
            const int l = i / kHid, c = i % kHid;
            sBias[i] = (l < kLayers - 1 || c < kOut) ? params[b_offset(l) + c] : 0.0f;
        }
    }
    if (threadIdx.x == 0) {
        for (int w = 0; w < kFwdWG; w++) mbar_init(bars + w, 1);
        barrier_init_fence();
    }
    if (warp == 0) {
        tmem_alloc(tslot, 512);
        tmem_relinquish();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tslot + 128u * g;
    uint64_t* bar = bars + g;
    uint32_t phase = 0;
    const int64_t n_tiles = (n + kTile - 1) / kTile;
    for (int64_t tile = static_cast<int64_t>(blockIdx.x) * kFwdWG + g; tile < n_tiles;
         tile += static_cast<int64_t>(gridDim.x) * kFwdWG) {
        const int64_t row = tile * kTile + t;
        const bool valid = row < n;
        {
            const uint4* xs = reinterpret_cast<const uint4*>(X + row * kIn0);
#pragma unroll
            for (int c = 0; c < kIn0 / 8; c++) {
                const uint4 v = valid ? xs[c] : make_uint4(0, 0, 0, 0);
                *reinterpret_cast<uint4*>(sH + kmajor_offset(t, 8 * c, kIn0)) = v;
            }
        }
        wg_sync_for_mma(bar_id);
        bool ok = true;
        for (int l = 0; l < kLayers; l++) {
            const int K = dim_in(l), N = dim_out(l);
            if (t == 0) {
                const uint32_t a = smem_addr(sH);
                const uint32_t b = smem_addr(sW) + static_cast<uint32_t>(fwd_img_offset(l) * 2);
                const uint32_t id = idesc_bf16_f32(128, N);
                for (int ks = 0; ks < K / 16; ks++)
                    mma_bf16(tmem, kslice_desc(a, K, ks), kslice_desc(b, K, ks), id, ks > 0);
                mma_commit(bar);
            }
            ok = wg_sync_and(bar_id, mbar_wait(bar, phase, err, 2));
            phase ^= 1u;
            if (!ok) break;
            fence_after_sync();
            const float* bias = params + b_offset(l);
            const float* sb = sBias + l * kHid;
            if (l < kLayers - 1) {
                // 64 columns per wait: two TMEM loads in flight at a time
                for (int c0 = 0; c0 < kHid; c0 += 64) {
                    uint32_t va[32], vb[32];
                    tmem_ld32_nowait(tmem_lane_addr(tmem, warp, c0), va);
                    tmem_ld32_nowait(tmem_lane_addr(tmem, warp, c0 + 32), vb);
                    tmem_wait_ld();
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        uint4 pk;
                        uint32_t* pw = reinterpret_cast<uint32_t*>(&pk);
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const int k = 8 * q + 2 * j;          // column within the 64
                            const uint32_t x0 = k < 32 ? va[k] : vb[k - 32];
                            const uint32_t x1 = k < 32 ? va[k + 1] : vb[k - 31];
                            pw[j] = pack_bf16x2(fmaxf(__uint_as_float(x0) + sb[c0 + k], 0.0f),
                                                fmaxf(__uint_as_float(x1) + sb[c0 + k + 1], 0.0f));
                        }
                        *reinterpret_cast<uint4*>(sH + kmajor_offset(t, c0 + 8 * q, kHid)) = pk;
                        if (acts && valid)
                            *reinterpret_cast<uint4*>(acts + (static_cast<int64_t>(l) * n + row) * kHid +
                                                      c0 + 8 * q) = pk;
                    }
                }
            } else if (records) {
                // fused epilogue: the row's mixture record, staged in the
                // warpgroup's buffer (free once the last GEMM has completed),
                // then stored for the whole tile with coalesced 16-byte stores
                float z[64];
                tmem_ld32(tmem_lane_addr(tmem, warp, 0), *reinterpret_cast<float(*)[32]>(z));
                tmem_ld32(tmem_lane_addr(tmem, warp, 32), *reinterpret_cast<float(*)[32]>(z + 32));
#pragma unroll
                for (int j = 0; j < kOutUsed; j++) z[j] += __ldg(bias + j);
                float* r = reinterpret_cast<float*>(sH) + t * kOut;
                mixture_record(z, r);
                wg_sync(bar_id);
                const int64_t rows = min(static_cast<int64_t>(kTile), n - tile * kTile);
                const float4* src = reinterpret_cast<const float4*>(sH);
                float4* dst = reinterpret_cast<float4*>(records + tile * kTile * kOut);
                for (int i = t; i < rows * (kOut / 4); i += 128) dst[i] = src[i];
            } else {
                for (int c0 = 0; c0 < kOut; c0 += 32) {
                    float v[32];
                    tmem_ld32(tmem_lane_addr(tmem, warp, c0), v);
                    if (valid) {
                        float4* o = reinterpret_cast<float4*>(out + row * kOut + c0);
#pragma unroll
                        for (int j = 0; j < 8; j++)
                            o[j] = make_float4(v[4 * j] + __ldg(bias + c0 + 4 * j),
                                               v[4 * j + 1] + __ldg(bias + c0 + 4 * j + 1),
                                               v[4 * j + 2] + __ldg(bias + c0 + 4 * j + 2),
                                               v[4 * j + 3] + __ldg(bias + c0 + 4 * j + 3));
                    }
                }
            }
            wg_sync_for_mma(bar_id);
        }
        if (!ok) break;
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(*tslot, 512);
}

// ---------------------------------------------------------------------------
// mixture negative log-likelihood and its gradient with respect to the
// outputs (mean over the n rows)

__device__ __forceinline__ float log_vmf_norm(float kappa) {
    // ln(kappa / (4 pi sinh kappa))
    const float l4pi = 2.5310242469692907f;
    if (kappa < 1e-3f) return -l4pi - kappa * kappa * (1.0f / 6.0f);
    return -l4pi - kappa + logf(2.0f * kappa) - logf(-expm1f(-2.0f * kappa));
}
// (coth kappa - 1 / kappa) / kappa
__device__ __forceinline__ float langevin_over_kappa(float kappa) {
    if (kappa < 1e-2f) return 1.0f / 3.0f - kappa * kappa * (1.0f / 45.0f);
    const float e = expf(-2.0f * kappa);
    return ((1.0f + e) / (1.0f - e) - 1.0f / kappa) / kappa;
}

__global__ void __launch_bounds__(256)
mlp_loss_kernel(const float* __restrict__ out, const float4* __restrict__ target, int64_t n,
                float inv_n, float* __restrict__ dout, double* __restrict__ loss_base,
                const int* __restrict__ step) {
    const int64_t row = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    float nll = 0.0f;
    if (row < n && !(target[row].x > 0.0f)) {
        // a row without a target (K <= 0) contributes nothing
        for (int j = 0; j < kOut; j++) dout[row * kOut + j] = 0.0f;
    } else if (row < n) {
        const float* z = out + row * kOut;
        const float4 tg = target[row];
        const float lK = logf(tg.x);
        float lmax = -INFINITY;
        for (int k = 0; k < kComp; k++) lmax = fmaxf(lmax, z[k]);
        float se = 0.0f;
        for (int k = 0; k < kComp; k++) se += expf(z[k] - lmax);
        const float lse_w = lmax + logf(se);
        float lc[kComp];
        float cmax = -INFINITY;
        const float half_l2pi = 0.91893853320467274f;
        for (int k = 0; k < kComp; k++) {
            const float s = fminf(fmaxf(z[16 + k], kLogSigMin), kLogSigMax);
            const float is2 = expf(-2.0f * s);
            const float d = lK - z[8 + k];
            const float vx = z[24 + 3 * k], vy = z[25 + 3 * k], vz = z[26 + 3 * k];
            const float kap = sqrtf(vx * vx + vy * vy + vz * vz);
            lc[k] = z[k] - lse_w - s - half_l2pi - 0.5f * d * d * is2 + log_vmf_norm(kap) +
                    vx * tg.y + vy * tg.z + vz * tg.w;
            cmax = fmaxf(cmax, lc[k]);
        }
        float sc = 0.0f;
        for (int k = 0; k < kComp; k++) sc += expf(lc[k] - cmax);
        const float L = cmax + logf(sc);
        nll = -(L - lK);
        float* g = dout + row * kOut;
        for (int k = 0; k < kComp; k++) {
            const float r = expf(lc[k] - L);
            const float w = expf(z[k] - lse_w);
            const float sraw = z[16 + k];
            const float s = fminf(fmaxf(sraw, kLogSigMin), kLogSigMax);
            const float is2 = expf(-2.0f * s);
            const float d = lK - z[8 + k];
            const float vx = z[24 + 3 * k], vy = z[25 + 3 * k], vz = z[26 + 3 * k];
            const float kap = sqrtf(vx * vx + vy * vy + vz * vz);
            const float gk = langevin_over_kappa(kap);
            g[k] = (w - r) * inv_n;
            g[8 + k] = -r * d * is2 * inv_n;
            g[16 + k] = (sraw > kLogSigMin && sraw < kLogSigMax) ? -r * (d * d * is2 - 1.0f) * inv_n : 0.0f;
            g[24 + 3 * k] = -r * (tg.y - gk * vx) * inv_n;
            g[25 + 3 * k] = -r * (tg.z - gk * vy) * inv_n;
            g[26 + 3 * k] = -r * (tg.w - gk * vz) * inv_n;
        }
        for (int j = kOutUsed; j < kOut; j++) g[j] = 0.0f;
    }
    // block sum of the loss
    __shared__ float s_part[8];
    float v = nll;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); w++) s += s_part[w];
        atomicAdd(step ? loss_base + *step : loss_base, s);
    }
}

// ---------------------------------------------------------------------------
// backward: parameter gradients of the mean loss, accumulated into grad
// (FP32, flat parameter layout) with atomics per tile

constexpr int kBwdSmem = 4 * kTile * kHid * 2 + 64;

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// stage 8 gradient values of row t at columns c..c+7 of a dZ tile with Kz
// columns: K-major copy sDZ[t][.] and transposed copy sDZt[c + j][t]
// (K = 128 rows of the tile); the bias gradient gets the column sums
__device__ __forceinline__ void stage_dz8(uint8_t* sDZ, uint8_t* sDZt, int t, int c, int Kz,
                                          const float (&d)[8], float* gbias) {
    uint4 pk;
    uint32_t* pw = reinterpret_cast<uint32_t*>(&pk);
#pragma unroll
    for (int j = 0; j < 4; j++) pw[j] = pack_bf16x2(d[2 * j], d[2 * j + 1]);
    *reinterpret_cast<uint4*>(sDZ + kmajor_offset(t, c, Kz)) = pk;
    const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(&pk);
#pragma unroll
    for (int j = 0; j < 8; j++)
        *reinterpret_cast<__nv_bfloat16*>(sDZt + kmajor_offset(c + j, t, kTile)) = hb[j];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const float s = warp_sum(d[j]);
        if ((t & 31) == 0 && s != 0.0f) atomicAdd(gbias + c + j, s);
    }
}

// transposed copy of row t of an activation tile: sHt[i][t] for i < width
__device__ __forceinline__ void stage_ht(uint8_t* sHt, int t, const __nv_bfloat16* src, int width,
                                         bool valid) {
    for (int c = 0; c < width; c += 8) {
        uint4 v = valid ? *reinterpret_cast<const uint4*>(src + c) : make_uint4(0, 0, 0, 0);
        const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(&v);
#pragma unroll
        for (int j = 0; j < 8; j++)
            *reinterpret_cast<__nv_bfloat16*>(sHt + kmajor_offset(c + j, t, kTile)) = hb[j];
    }
}

__global__ void __launch_bounds__(128, 1)
mlp_bwd_kernel(const __nv_bfloat16* __restrict__ img, const __nv_bfloat16* __restrict__ X,
               const __nv_bfloat16* __restrict__ acts, const float* __restrict__ dout, int64_t n,
               float* __restrict__ grad, int* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sWt = smem;
    uint8_t* sDZ = sWt + kTile * kHid * 2;
    uint8_t* sDZt = sDZ + kTile * kHid * 2;
    uint8_t* sHt = sDZt + kTile * kHid * 2;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sHt + kTile * kHid * 2);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    const int t = threadIdx.x, warp = t >> 5;
    if (t == 0) {
        mbar_init(bar, 1);
        barrier_init_fence();
    }
    if (warp == 0) {
        tmem_alloc(tslot, 256);
        tmem_relinquish();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t tm_dh = tmem, tm_dw = tmem + 128;
    uint32_t phase = 0;
    bool ok = true;
    const int64_t n_tiles = (n + kTile - 1) / kTile;
    for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const int64_t row = tile * kTile + t;
        const bool valid = row < n;
        // dZ of the output layer from the loss gradient
        for (int c = 0; c < kOut; c += 8) {
            float d[8];
#pragma unroll
            for (int j = 0; j < 8; j++) d[j] = valid ? dout[row * kOut + c + j] : 0.0f;
            stage_dz8(sDZ, sDZt, t, c, kOut, d, grad + b_offset(kLayers - 1));
        }
        for (int l = kLayers - 1; l >= 0; l--) {
            const int K_in = dim_in(l), K_out = dim_out(l);
            // input of layer l, transposed
            if (l == 0)
                stage_ht(sHt, t, X + row * kIn0, kIn0, valid);
            else
                stage_ht(sHt, t, acts + (static_cast<int64_t>(l - 1) * n + row) * kHid, kHid, valid);
            if (l > 0) {
                const uint4* src = reinterpret_cast<const uint4*>(img + bwd_img_offset(l));
                uint4* dst = reinterpret_cast<uint4*>(sWt);
                for (int i = t; i < K_in * K_out * 2 / 16; i += 128) dst[i] = src[i];
            }
            sync_for_mma();
            if (t == 0) {
                if (l > 0) {
                    // dH[b][i] = sum_o dZ[b][o] W[o][i]
                    const uint32_t id = idesc_bf16_f32(128, K_in);
                    for (int ks = 0; ks < K_out / 16; ks++)
                        mma_bf16(tm_dh, kslice_desc(smem_addr(sDZ), K_out, ks),
                                 kslice_desc(smem_addr(sWt), K_out, ks), id, ks > 0);
                }
                if (l == kLayers - 1) {
                    // dW^T[i][o] = sum_b H[b][i] dZ[b][o]
                    const uint32_t id = idesc_bf16_f32(128, K_out);
                    for (int ks = 0; ks < kTile / 16; ks++)
                        mma_bf16(tm_dw, kslice_desc(smem_addr(sHt), kTile, ks),
                                 kslice_desc(smem_addr(sDZt), kTile, ks), id, ks > 0);
                } else {
                    // dW[o][i] = sum_b dZ[b][o] H[b][i]
                    const uint32_t id = idesc_bf16_f32(128, K_in);
                    for (int ks = 0; ks < kTile / 16; ks++)
                        mma_bf16(tm_dw, kslice_desc(smem_addr(sDZt), kTile, ks),
                                 kslice_desc(smem_addr(sHt), kTile, ks), id, ks > 0);
                }
                mma_commit(bar);
            }
            ok = __syncthreads_and(mbar_wait(bar, phase, err, 3));
            phase ^= 1u;
            if (!ok) break;
            fence_after_sync();
            // weight gradient
            float* gw = grad + w_offset(l);
            if (l == kLayers - 1) {
                for (int c0 = 0; c0 < K_out; c0 += 32) {
                    float v[32];
                    tmem_ld32(tmem_lane_addr(tm_dw, warp, c0), v);
#pragma unroll
                    for (int j = 0; j < 32; j++)
                        if (v[j] != 0.0f) atomicAdd(gw + (c0 + j) * K_in + t, v[j]);
                }
            } else {
                for (int c0 = 0; c0 < K_in; c0 += 32) {
                    float v[32];
                    tmem_ld32(tmem_lane_addr(tm_dw, warp, c0), v);
#pragma unroll
                    for (int j = 0; j < 32; j++)
                        if (v[j] != 0.0f) atomicAdd(gw + t * K_in + c0 + j, v[j]);
                }
            }
            // dZ of layer l - 1: dH masked by the ReLU of H_{l-1}
            if (l > 0) {
                const __nv_bfloat16* h = acts + (static_cast<int64_t>(l - 1) * n + row) * kHid;
                for (int c0 = 0; c0 < kHid; c0 += 32) {
                    float v[32];
                    tmem_ld32(tmem_lane_addr(tm_dh, warp, c0), v);
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        uint4 hv = valid ? *reinterpret_cast<const uint4*>(h + c0 + 8 * q)
                                         : make_uint4(0, 0, 0, 0);
                        const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(&hv);
                        float d[8];
#pragma unroll
                        for (int j = 0; j < 8; j++)
                            d[j] = __bfloat162float(hb[j]) > 0.0f ? v[8 * q + j] : 0.0f;
                        stage_dz8(sDZ, sDZt, t, c0 + 8 * q, kHid, d, grad + b_offset(l - 1));
                    }
                }
            }
            fence_before_sync();
            __syncthreads();
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 256);
}

// ---------------------------------------------------------------------------
// Adam on the FP32 masters; refreshes the bf16 images and clears the gradient

__global__ void mlp_adam_kernel(float* __restrict__ params, float* __restrict__ m1,
                                float* __restrict__ m2, float* __restrict__ grad,
                                __nv_bfloat16* __restrict__ img, const int* __restrict__ step,
                                float lr, float b1, float b2, float eps) {
    const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= kNumParams) return;
    const float g = grad[p];
    grad[p] = 0.0f;
    const int s = *step + 1;
    const float a = b1 * m1[p] + (1.0f - b1) * g;
    const float b = b2 * m2[p] + (1.0f - b2) * g * g;
    m1[p] = a;
    m2[p] = b;
    const float bc1 = 1.0f - powf(b1, static_cast<float>(s));
    const float bc2 = 1.0f - powf(b2, static_cast<float>(s));
    const float w = params[p] - lr * (a / bc1) / (sqrtf(b / bc2) + eps);
    params[p] = w;
    int l = 0;
    while (l < kLayers - 1 && p >= w_offset(l + 1)) l++;
    const int64_t q = p - w_offset(l);
    const int K_in = dim_in(l), K_out = dim_out(l);
    if (q < static_cast<int64_t>(K_in) * K_out) {
        const int o = static_cast<int>(q / K_in), i = static_cast<int>(q % K_in);
        const __nv_bfloat16 wb = __float2bfloat16_rn(w);
        img[fwd_img_offset(l) + kmajor_offset(o, i, K_in) / 2] = wb;
        if (l > 0) img[bwd_img_offset(l) + kmajor_offset(i, o, K_out) / 2] = wb;
    }
}

__global__ void step_advance_kernel(int* step) { *step += 1; }

// bf16 images of the FP32 masters (weights set from the host)
__global__ void mlp_images_kernel(const float* __restrict__ params, __nv_bfloat16* __restrict__ img) {
    const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= kNumParams) return;
    int l = 0;
    while (l < kLayers - 1 && p >= w_offset(l + 1)) l++;
    const int64_t q = p - w_offset(l);
    const int K_in = dim_in(l), K_out = dim_out(l);
    if (q < static_cast<int64_t>(K_in) * K_out) {
        const int o = static_cast<int>(q / K_in), i = static_cast<int>(q % K_in);
        const __nv_bfloat16 wb = __float2bfloat16_rn(params[p]);
        img[fwd_img_offset(l) + kmajor_offset(o, i, K_in) / 2] = wb;
        if (l > 0) img[bwd_img_offset(l) + kmajor_offset(i, o, K_out) / 2] = wb;
    }
}

// FP32 features [n][18] -> bf16 [n][32] (zero-padded)
__global__ void features_to_bf16_kernel(const float* __restrict__ f, int64_t n,
                                        __nv_bfloat16* __restrict__ x) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n * kIn0) return;
    const int64_t r = i / kIn0;
    const int c = static_cast<int>(i % kIn0);
    x[i] = __float2bfloat16_rn(c < kFeatures ? f[r * kFeatures + c] : 0.0f);
}

// a training batch drawn with replacement: row r of step s takes sample
// floor(u * n_data) with u from Philox (counter (s, r, 0, tag))
__global__ void gather_batch_kernel(const __nv_bfloat16* __restrict__ data_x,
                                    const float4* __restrict__ data_t, int64_t n_data,
                                    const int* __restrict__ step, uint32_t key0, uint32_t key1,
                                    int64_t batch, __nv_bfloat16* __restrict__ x,
                                    float4* __restrict__ tg) {
    const int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= batch) return;
    const uint4 w = philox4x32_10(make_uint4(static_cast<uint32_t>(*step), static_cast<uint32_t>(r),
                                             0u, 0x4C524E00u), key0, key1);
    const unsigned long long u = (static_cast<unsigned long long>(w.x) << 32) | w.y;
    const int64_t j = static_cast<int64_t>(__umul64hi(u, static_cast<unsigned long long>(n_data)));
    const uint4* src = reinterpret_cast<const uint4*>(data_x + j * kIn0);
    uint4* dst = reinterpret_cast<uint4*>(x + r * kIn0);
#pragma unroll
    for (int c = 0; c < kIn0 / 8; c++) dst[c] = src[c];
    tg[r] = data_t[j];
}

// dynamic shared memory above 48 KB is opted into once per kernel and device
// (outside of any stream capture: the first call of a wrapper is eager)
template <typename K>
cudaError_t smem_opt_in(K kernel, int bytes, unsigned long long* done_mask) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (*done_mask & bit) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) *done_mask |= bit;
    return e;
}
unsigned long long g_fwd_attr = 0, g_bwd_attr = 0;

}  // namespace

// ---------------------------------------------------------------------------
// launch wrappers

cudaError_t launch_mma_selftest(const void* A, const void* B, int N, int K, float* C, int* err,
                                cudaStream_t s) {
    uint32_t ncols = 32;
    while (static_cast<int>(ncols) < N) ncols <<= 1;
    const int smem = 128 * K * 2 + N * K * 2 + 64;
    cudaError_t e = cudaFuncSetAttribute(mma_selftest_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    mma_selftest_kernel<<<1, 128, smem, s>>>(static_cast<const __nv_bfloat16*>(A),
                                             static_cast<const __nv_bfloat16*>(B), N, K, ncols, C,
                                             err);
    return cudaGetLastError();
}

cudaError_t launch_mlp_images(const float* params, void* img, cudaStream_t s) {
    mlp_images_kernel<<<static_cast<unsigned>((kNumParams + 255) / 256), 256, 0, s>>>(
        params, static_cast<__nv_bfloat16*>(img));
    return cudaGetLastError();
}

cudaError_t launch_features_to_bf16(const float* f, int64_t n, void* x, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    features_to_bf16_kernel<<<static_cast<unsigned>((n * kIn0 + 255) / 256), 256, 0, s>>>(
        f, n, static_cast<__nv_bfloat16*>(x));
    return cudaGetLastError();
}

cudaError_t launch_mlp_forward(const void* img, const float* params, const void* X, int64_t n,
                               float* out, void* acts, int* err, int num_sms, cudaStream_t s,
                               float* records) {
    if (n <= 0) return cudaSuccess;
    cudaError_t e = smem_opt_in(mlp_fwd_kernel, kFwdSmem, &g_fwd_attr);
    if (e != cudaSuccess) return e;
    const int64_t groups = (n + kTile * kFwdWG - 1) / (kTile * kFwdWG);
    const int grid = static_cast<int>(groups < num_sms ? groups : num_sms);
    mlp_fwd_kernel<<<grid, kFwdThreads, kFwdSmem, s>>>(static_cast<const __nv_bfloat16*>(img), params,
                                               static_cast<const __nv_bfloat16*>(X), n, out,
                                               static_cast<__nv_bfloat16*>(acts), records, err);
    return cudaGetLastError();
}

cudaError_t launch_mlp_loss(const float* out, const void* target, int64_t n, float* dout,
                            double* loss_base, const int* step, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    mlp_loss_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(
        out, static_cast<const float4*>(target), n, 1.0f / static_cast<float>(n), dout, loss_base,
        step);
    return cudaGetLastError();
}

cudaError_t launch_mlp_backward(const void* img, const void* X, const void* acts, const float* dout,
                                int64_t n, float* grad, int* err, int num_sms, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    cudaError_t e = smem_opt_in(mlp_bwd_kernel, kBwdSmem, &g_bwd_attr);
    if (e != cudaSuccess) return e;
    const int64_t tiles = (n + kTile - 1) / kTile;
    const int grid = static_cast<int>(tiles < num_sms ? tiles : num_sms);
    mlp_bwd_kernel<<<grid, 128, kBwdSmem, s>>>(static_cast<const __nv_bfloat16*>(img),
                                               static_cast<const __nv_bfloat16*>(X),
                                               static_cast<const __nv_bfloat16*>(acts), dout, n, grad,
                                               err);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float* params, float* m1, float* m2, float* grad, void* img,
                            const int* step, float lr, float b1, float b2, float eps,
                            cudaStream_t s) {
    mlp_adam_kernel<<<static_cast<unsigned>((kNumParams + 255) / 256), 256, 0, s>>>(
        params, m1, m2, grad, static_cast<__nv_bfloat16*>(img), step, lr, b1, b2, eps);
    return cudaGetLastError();
}

cudaError_t launch_step_advance(int* step, cudaStream_t s) {
    step_advance_kernel<<<1, 1, 0, s>>>(step);
    return cudaGetLastError();
}

cudaError_t launch_gather_batch(const void* data_x, const void* data_t, int64_t n_data,
                                const int* step, uint32_t key0, uint32_t key1, int64_t batch,
                                void* x, void* tg, cudaStream_t s) {
    if (batch <= 0 || n_data <= 0) return cudaSuccess;
    gather_batch_kernel<<<static_cast<unsigned>((batch + 255) / 256), 256, 0, s>>>(
        static_cast<const __nv_bfloat16*>(data_x), static_cast<const float4*>(data_t), n_data, step,
        key0, key1, batch, static_cast<__nv_bfloat16*>(x), static_cast<float4*>(tg));
    return cudaGetLastError();
}

}  // namespace iss
