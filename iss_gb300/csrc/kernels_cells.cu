// Per-cell kernels of the sampling path:
//   yields_kernel         FSSW::calculate_dN_dxtdy_for_one_particle_species
//                         + calculate_dN_analytic (src/FSSW.cpp:565-848) for every
//                           (cell, species) pair
//   cdf kernels           RandomVariable1DArray (src/RandomVariable1DArray.cpp:25-74):
//                         per-species FP64 prefix sums of the cell yields
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "kernels.h"

namespace iss {

namespace {

constexpr float kHbarCf = 0.197327053f;

// ------------------------------------------------------------------------
// special functions off the table (x < 0.5 or x > 399.95): direct
// evaluation of K_n from its integral representation (trapezoidal rule)
__device__ double bessel_k_direct(int n, double x) {
    if (x > 700.0) return 0.0;
    const double h = fmin(0.02, 0.5 / sqrt(x));
    double acc = 0.5;
    for (int k = 1; k < 20000; k++) {
        const double t = k * h;
        const double lg = n * t - x * (cosh(t) - 1.0);
        acc += 0.5 * exp(lg) * (1.0 + exp(-2.0 * n * t));
        if (lg < -70.0) break;
    }
    return acc * h * exp(-x);
}

__device__ double expint_direct(int n, double x) {
    if (x > 1.0) {
        double b = x + n, c = 1e300, d = 1.0 / b, h = d;
        for (int i = 1; i < 10000; i++) {
            const double a = -static_cast<double>(i) * (n - 1 + i);
            b += 2.0;
            d = 1.0 / (a * d + b);
            c = b + a / c;
            const double del = c * d;
            h *= del;
            if (fabs(del - 1.0) < 1e-16) break;
        }
        return h * exp(-x);
    }
    const double ge = 0.57721566490153286061;
    double psi = -ge;
    for (int k = 1; k < n; k++) psi += 1.0 / k;
    double sum = (n == 1) ? (-log(x) - ge) : 1.0 / (n - 1);
    double term = 1.0;
    for (int m = 1; m < 500; m++) {
        term *= -x / m;
        const double del = (m != n - 1) ? -term / (m - n + 1) : term * (psi - log(x));
        sum += del;
        if (fabs(del) < 1e-17 * fabs(sum)) break;
    }
    return sum;
}

// Position of a float-float argument on the special-function grid.
struct GridPos {
    int idx;
    float frac;
    bool on_table;
};

__device__ __forceinline__ GridPos grid_pos(float xh, float xl) {
    GridPos g;
    g.on_table = (xh >= 0.5f) && (xh <= 399.95f);
    float s, se;
    two_sum(xh, -0.5f, s, se);
    se += xl;
    float ph, pe;
    two_prod(s, 20.0f, ph, pe);
    const float pl = fmaf(20.0f, se, pe);
    int idx = static_cast<int>(floorf(ph));
    float f = (ph - static_cast<float>(idx)) + pl;
    if (f < 0.0f) {
        idx -= 1;
        f += 1.0f;
    } else if (f >= 1.0f) {
        idx += 1;
        f -= 1.0f;
    }
    g.idx = min(max(idx, 0), 7989);
    g.frac = f;
    return g;
}

// ------------------------------------------------------------------------
constexpr int kYieldThreads = 128;

__global__ void __launch_bounds__(kYieldThreads)
yields_kernel(DevConfig cfg, CellArrays cells, const SpeciesDev* __restrict__ species,
              float* __restrict__ yields) {
    extern __shared__ SpeciesDev s_sp[];
    const int nsp = cfg.n_species;
    for (int k = threadIdx.x; k < nsp; k += blockDim.x) s_sp[k] = species[k];
    __syncthreads();
    const int64_t n = cfg.n_cells;
    const int64_t l = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (l >= n) return;

    const float4 da = cells.da[l];
    if (da.x < 0.0f) {
        for (int k = 0; k < nsp; k++) yields[static_cast<int64_t>(k) * n + l] = 0.0f;
        return;
    }
    const float4 th = cells.th[l];
    const float4 th2 = cells.th2[l];
    const float4 cf = cells.coef[l];
    const float T = th.x;
    const double beta_d = 1.0 / static_cast<double>(T);
    const float b_hi = static_cast<float>(beta_d);
    const float b_lo = static_cast<float>(beta_d - static_cast<double>(b_hi));
    const bool warm = static_cast<double>(T) > 0.05;
    const int bulk_kind = cfg.bulk_kind;
    const bool with_bulk = cfg.include_bulk != 0;
    const bool with_diff = cfg.include_diff != 0;
    const bool kind_ce = (bulk_kind == 1 || bulk_kind == 21);
    const bool kind_14 = (bulk_kind == 11 || bulk_kind == 20);
    float bulkPi = 0.0f;
    if (with_bulk) bulkPi = (bulk_kind == 21 || bulk_kind == 20 || bulk_kind == 11 || bulk_kind == 0)
                                ? th2.w : th2.w / kHbarCf;
    float dsq = 0.0f, pref_q = 0.0f, inv_kappa = 0.0f;
    if (with_diff) {
        const float4 p2 = cells.pi2[l];
        dsq = p2.y * da.y + p2.z * da.z + p2.w * da.w;
        pref_q = th2.z / (th2.x + th2.y);
        inv_kappa = 1.0f / cf.w;
    }
    // (1/hbarc^3) / (2 pi^2)
    const float unit_pref = (1.0f / (0.197327053f * 0.197327053f * 0.197327053f)) /
                            (2.0f * 9.8696044010893586f);

    for (int k = 0; k < nsp; k++) {
        const SpeciesDev sp = s_sp[k];
        const float mass = sp.m_hi + sp.m_lo;
        const float mu = static_cast<float>(sp.baryon) * th.y + static_cast<float>(sp.strange) * th.z +
                         static_cast<float>(sp.charge) * th.w;
        // beta*mu and m*beta as float-float numbers
        float bm_h, bm_e;
        two_prod(mu, b_hi, bm_h, bm_e);
        const float bm_l = fmaf(mu, b_lo, bm_e);
        float x1_h, x1_e;
        two_prod(sp.m_hi, b_hi, x1_h, x1_e);
        const float x1_l = x1_e + fmaf(sp.m_hi, b_lo, sp.m_lo * b_hi);
        const int nmax = (sp.light && warm) ? 10 : 1;
        float Neq = 0.f, b1 = 0.f, b2 = 0.f, b3 = 0.f, q1 = 0.f, q2 = 0.f;
        const float mbeta = x1_h + x1_l;
        for (int nn = 1; nn <= nmax; nn++) {
            const float fn = static_cast<float>(nn);
            float theta = 1.0f;
            if (sp.sign == 1 && (nn % 2 == 0)) theta = -1.0f;
            if (sp.sign == 0 && nn > 1) theta = 0.0f;
            // x_n = n m beta
            float xh, xe;
            two_prod(fn, x1_h, xh, xe);
            const float xl = fmaf(fn, x1_l, xe);
            // lambda^n = exp(n beta mu)
            float ah, ae;
            two_prod(fn, bm_h, ah, ae);
            const float al = fmaf(fn, bm_l, ae);
            const float fug = expf(ah) * (1.0f + al);
            const GridPos g = grid_pos(xh, xl);
            float K1, K2, K3;
            if (g.on_table) {
                const float4 ka = __ldg(cfg.tab.sfK + g.idx);
                const float4 kb = __ldg(cfg.tab.sfK + g.idx + 1);
                K1 = fmaf(g.frac, kb.x - ka.x, ka.x);
                K2 = fmaf(g.frac, kb.y - ka.y, ka.y);
                K3 = fmaf(g.frac, kb.z - ka.z, ka.z);
            } else {
                const double xd = static_cast<double>(xh) + static_cast<double>(xl);
                K2 = static_cast<float>(bessel_k_direct(2, xd));
                K1 = with_bulk ? static_cast<float>(bessel_k_direct(1, xd)) : 0.0f;
                K3 = (with_bulk && kind_14) ? static_cast<float>(bessel_k_direct(3, xd)) : 0.0f;
            }
            const float tf = theta * fug;
            Neq = fmaf(tf / fn, K2, Neq);
            if (with_bulk) {
                if (kind_ce) {
                    b1 = fmaf(tf, fmaf(mbeta, K1, 3.0f * K2 / fn), b1);
                    b2 = fmaf(tf, K1, b2);
                } else if (kind_14) {
                    b1 = fmaf(tf, K2, b1);
                    b2 = fmaf(tf, fmaf(mbeta, K1, 3.0f * K2 / fn), b2);
                    b3 = fmaf(tf, fmaf(mbeta, K2, 3.0f * K3 / fn), b3);
                }
            }
            if (with_diff) {
                q1 = fmaf(tf / fn, K2, q1);
                float En[9];
                if (g.on_table) {
                    const float* ea = cfg.tab.sfE + 9 * g.idx;
#pragma unroll
                    for (int i = 0; i < 9; i++) {
                        const float a = __ldg(ea + i), b = __ldg(ea + 9 + i);
                        En[i] = fmaf(g.frac, b - a, a);
                    }
                } else {
                    const double xd = static_cast<double>(xh) + static_cast<double>(xl);
                    En[0] = static_cast<float>(expint_direct(2, xd));
                    for (int i = 1; i < 9; i++) En[i] = static_cast<float>(expint_direct(2 * i + 2, xd));
                }
                const float arg = xh;
                const float em = expf(-xh) * (1.0f - xl);
                float I = em / arg * (2.0f / (arg * arg) + 2.0f / arg - 0.5f) + 0.375f * En[0];
                // 3 (2k-5)!! / (2^k k!) for k = 3..10
                const float ck[8] = {0.0625f, 0.0234375f, 0.01171875f, 0.0068359375f,
                                     0.00439453125f, 0.0030212402343750f,
                                     0.0021820068359375f, 0.0016365051269531f};
#pragma unroll
                for (int k2 = 0; k2 < 8; k2++) I = fmaf(ck[k2], En[k2 + 1], I);
                I = -(mbeta * mbeta * mbeta) * I;
                q2 = fmaf(fn * tf, I, q2);
            }
        }
        const float m2 = mass * mass;
        const float ug = unit_pref * sp.degen;
        const float pref = ug * da.x;
        float total = pref * (m2 * T * Neq);
        if (with_bulk) {
            if (kind_ce) {
                // Chapman-Enskog form, bulk_deltaf_kind 1 and 21
                const float r1 = m2 * T * b1;
                const float r2 = m2 * mass / 3.0f * b2;
                total += pref * (-bulkPi * cf.x) * (-cf.y * r1 + r2);
            } else if (bulk_kind == 11) {
                const float r1 = m2 * T * b1;
                const float r2 = m2 * T * T * b2;
                const float r3 = m2 * mass * T * T * b3;
                total += pref * bulkPi *
                         (r1 * m2 * cf.x + r2 * static_cast<float>(sp.baryon) * cf.y + r3 * cf.z);
            }
        }
        if (with_diff) {
            const float r4 = m2 * T * T * q1;
            const float r5 = (T * T * T / 3.0f) * q2;
            total += ug * dsq * inv_kappa * (-pref_q * r4 - static_cast<float>(sp.baryon) * r5);
        }
        yields[static_cast<int64_t>(k) * n + l] = fmaxf(total, 0.0f);
    }
}

// ------------------------------------------------------------------------
// per-species FP64 prefix sums over cells: tile sums, tile offsets, tile scan

constexpr int kScanThreads = 256;
constexpr int kScanPer = 16;
constexpr int kScanTile = kScanThreads * kScanPer;

__device__ __forceinline__ double warp_incl_scan(double v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// exclusive block scan of one double per thread; returns the block total
__device__ double block_excl_scan(double v, double* s_warp, double* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const double inc = warp_incl_scan(v);
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        double w = lane < nw ? s_warp[lane] : 0.0;
        const double wi = warp_incl_scan(w);
        if (lane < nw) s_warp[lane] = wi - w;
        if (lane == nw - 1) s_warp[32] = wi;
    }
    __syncthreads();
    const double out = s_warp[wid] + inc - v;
    *total = s_warp[32];
    __syncthreads();
    return out;
}

__global__ void __launch_bounds__(kScanThreads)
cdf_tile_sum_kernel(const float* __restrict__ yields, int64_t n, int n_tiles,
                    double* __restrict__ tile_sum) {
    __shared__ double s_warp[33];
    const int s = blockIdx.y;
    const int64_t t0 = static_cast<int64_t>(blockIdx.x) * kScanTile;
    const float* row = yields + static_cast<int64_t>(s) * n;
    double acc = 0.0;
    for (int k = 0; k < kScanPer; k++) {
        const int64_t i = t0 + k * kScanThreads + threadIdx.x;
        if (i < n) acc += static_cast<double>(fmaxf(row[i], 0.0f));
    }
    double tot;
    block_excl_scan(acc, s_warp, &tot);
    if (threadIdx.x == 0) tile_sum[static_cast<int64_t>(s) * n_tiles + blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads)
cdf_tile_offset_kernel(const double* __restrict__ tile_sum, int n_tiles, int64_t n, int guide_len,
                       double* __restrict__ tile_off, double* __restrict__ totals,
                       int32_t* __restrict__ guide) {
    __shared__ double s_warp[33];
    const int s = blockIdx.x;
    double carry = 0.0;
    for (int b = 0; b < n_tiles; b += kScanThreads) {
        const int i = b + threadIdx.x;
        const double v = i < n_tiles ? tile_sum[static_cast<int64_t>(s) * n_tiles + i] : 0.0;
        double tot;
        const double ex = block_excl_scan(v, s_warp, &tot);
        if (i < n_tiles) tile_off[static_cast<int64_t>(s) * n_tiles + i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        totals[s] = carry;
        int32_t* g = guide + static_cast<int64_t>(s) * (guide_len + 1);
        g[0] = 0;
        g[guide_len] = static_cast<int32_t>(n - 1);
    }
}

// Writes the FP64 CDF row of species s and scatters its guide table
// (indexed search, Chen & Asau 1974): bucket j of guide_len covers
// v in [j, j+1) * total / guide_len and guide[j] is the cell whose CDF
// interval contains the bucket's left edge, so the cell of any v in bucket j
// lies in [guide[j], guide[j+1]].  Entries at tile seams may stay unset (-1);
// the sampler then falls back to a full binary search.
__global__ void __launch_bounds__(kScanThreads)
cdf_tile_scan_kernel(const float* __restrict__ yields, int64_t n, int n_tiles,
                     const double* __restrict__ tile_off, const double* __restrict__ totals,
                     int guide_len, double* __restrict__ cdf, int32_t* __restrict__ guide) {
    __shared__ float s_in[kScanThreads * (kScanPer + 1)];
    __shared__ double s_warp[33];
    __shared__ double s_last[kScanThreads];
    const int s = blockIdx.y;
    const int64_t t0 = static_cast<int64_t>(blockIdx.x) * kScanTile;
    const float* row = yields + static_cast<int64_t>(s) * n;
    double* out = cdf + static_cast<int64_t>(s) * (n + 1);
    int32_t* g = guide + static_cast<int64_t>(s) * (guide_len + 1);
    // coalesced load into a padded layout: element e -> (e / 16) * 17 + e % 16
    for (int k = 0; k < kScanPer; k++) {
        const int e = k * kScanThreads + threadIdx.x;
        const int64_t i = t0 + e;
        s_in[(e / kScanPer) * (kScanPer + 1) + e % kScanPer] = i < n ? fmaxf(row[i], 0.0f) : 0.0f;
    }
    __syncthreads();
    const float* mine = s_in + threadIdx.x * (kScanPer + 1);
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) acc += static_cast<double>(mine[k]);
    double tot;
    const double ex = block_excl_scan(acc, s_warp, &tot);
    const double base = tile_off[static_cast<int64_t>(s) * n_tiles + blockIdx.x];
    double run = base + ex;
    double vals[kScanPer];
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
        run += static_cast<double>(mine[k]);
        vals[k] = run;
    }
    s_last[threadIdx.x] = run;
    __syncthreads();
    const int64_t e0 = t0 + static_cast<int64_t>(threadIdx.x) * kScanPer;
    // value written just before this thread's first element
    double prev = threadIdx.x == 0 ? base : s_last[threadIdx.x - 1];
    const double total = totals[s];
    const double scale = total > 0.0 ? static_cast<double>(guide_len) / total : 0.0;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
        const int64_t i = e0 + k;
        if (i < n) {
            out[i + 1] = vals[k];
            if (scale > 0.0 && vals[k] > prev) {
                int64_t jl = static_cast<int64_t>(floor(prev * scale)) + 1;
                int64_t jh = static_cast<int64_t>(floor(vals[k] * scale));
                jl = max(jl, static_cast<int64_t>(1));
                jh = min(jh, static_cast<int64_t>(guide_len - 1));
                for (int64_t j = jl; j <= jh; j++) g[j] = static_cast<int32_t>(i);
            }
        }
        prev = vals[k];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[0] = 0.0;
}

}  // namespace

// ------------------------------------------------------------------------
// launch wrappers

cudaError_t launch_yields(const DevConfig& cfg, const CellArrays& cells, const SpeciesDev* sp,
                          float* yields, cudaStream_t stream) {
    if (cfg.n_cells <= 0) return cudaSuccess;
    const unsigned blocks = static_cast<unsigned>((cfg.n_cells + kYieldThreads - 1) / kYieldThreads);
    const size_t smem = sizeof(SpeciesDev) * static_cast<size_t>(cfg.n_species);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(yields_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    yields_kernel<<<blocks, kYieldThreads, smem, stream>>>(cfg, cells, sp, yields);
    return cudaGetLastError();
}

int cdf_num_tiles(int64_t n) { return static_cast<int>((n + kScanTile - 1) / kScanTile); }

int cdf_guide_len(int64_t n) { return static_cast<int>(n < 4 ? 1 : (n + 3) / 4); }

cudaError_t launch_cdf(const float* yields, int n_species, int64_t n, double* tile_sum,
                       double* tile_off, double* totals, double* cdf, int32_t* guide,
                       cudaStream_t stream) {
    const int nt = cdf_num_tiles(n);
    if (nt == 0 || n_species == 0) return cudaSuccess;
    const int glen = cdf_guide_len(n);
    cudaError_t e = cudaMemsetAsync(guide, 0xFF,
                                    sizeof(int32_t) * static_cast<size_t>(glen + 1) * n_species,
                                    stream);
    if (e != cudaSuccess) return e;
    dim3 grid(static_cast<unsigned>(nt), static_cast<unsigned>(n_species));
    cdf_tile_sum_kernel<<<grid, kScanThreads, 0, stream>>>(yields, n, nt, tile_sum);
    cdf_tile_offset_kernel<<<n_species, kScanThreads, 0, stream>>>(tile_sum, nt, n, glen, tile_off,
                                                                   totals, guide);
    cdf_tile_scan_kernel<<<grid, kScanThreads, 0, stream>>>(yields, n, nt, tile_off, totals, glen,
                                                           cdf, guide);
    return cudaGetLastError();
}

}  // namespace iss
