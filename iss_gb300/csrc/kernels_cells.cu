// Per-cell kernels of the sampling path:
//   yields_kernel         FSSW::calculate_dN_dxtdy_for_one_particle_species
//                         + calculate_dN_analytic (src/FSSW.cpp:565-848) for every
//                           (cell, species) pair
//   cdf kernels           RandomVariable1DArray (src/RandomVariable1DArray.cpp:25-74):
//                         per-species fixed-point prefix sums of the cell yields
#include <cuda_runtime.h>

#include <algorithm>

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
constexpr int kYieldGroups = 4;   // species groups per cell (grid y)

// Surface of cell l in a batch: the last b with surf[b].c0 <= l.
__device__ __forceinline__ int surface_of(const SurfSeg* __restrict__ surf, int n_surf, int64_t l) {
    int lo = 0, hi = n_surf - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (surf[mid].c0 <= l) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Per-cell quantities shared by every species' yield in cell l.
struct CellYieldIn {
    float T, b_hi, b_lo;
    bool warm, with_bulk, kind_ce, kind_14;
    int bulk_kind;
    float bulkPi, dsq, pref_q, inv_kappa, unit_pref;
    float4 th, th2, cf;
};

// Sums of the thermal series (calculate_dN_analytic, src/FSSW.cpp:719-848) of
// one species in one cell: they depend on the species only through its
// float-float mass, statistics, number of terms and chemical potential mu.
struct SeriesSums {
    float Neq, b1, b2, b3, q1, q2;
};

__device__ __forceinline__ float species_mu(const SpeciesDev& sp, const float4& th) {
    return static_cast<float>(sp.baryon) * th.y + static_cast<float>(sp.strange) * th.z +
           static_cast<float>(sp.charge) * th.w;
}

template <bool kDiff>
__device__ __forceinline__ SeriesSums thermal_series(const DevConfig& cfg, const CellYieldIn& c,
                                                     const SpeciesDev& sp, float mu) {
    const float b_hi = c.b_hi, b_lo = c.b_lo;
    const bool warm = c.warm, with_bulk = c.with_bulk;
    constexpr bool with_diff = kDiff;
    const bool kind_ce = c.kind_ce, kind_14 = c.kind_14;
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
    return SeriesSums{Neq, b1, b2, b3, q1, q2};
}

// The yield of calculate_dN_dxtdy_for_one_particle_species
// (src/FSSW.cpp:565-715) is, for a species of degeneracy g and baryon number
// B, g (X + B Y): X and Y hold the prefactor, the equilibrium sum and the
// bulk and diffusion terms, and depend on the species only through the
// quantities its group shares (mass and the series sums).  They are formed
// once per series; each member then costs one multiply-add.
template <bool kDiff>
__device__ __forceinline__ float2 yield_coefs(const CellYieldIn& c, const SpeciesDev& sp,
                                              const SeriesSums& ss, float4 da) {
    const float T = c.T;
    const float4 cf = c.cf;
    const float mass = sp.m_hi + sp.m_lo;
    const float m2 = mass * mass;
    float x = m2 * T * ss.Neq;
    float y = 0.0f;
    if (c.with_bulk) {
        if (c.kind_ce) {
            // Chapman-Enskog form, bulk_deltaf_kind 1 and 21
            const float r1 = m2 * T * ss.b1;
            const float r2 = m2 * mass / 3.0f * ss.b2;
            x += (-c.bulkPi * cf.x) * (-cf.y * r1 + r2);
        } else if (c.bulk_kind == 11) {
            const float r1 = m2 * T * ss.b1;
            const float r2 = m2 * T * T * ss.b2;
            const float r3 = m2 * mass * T * T * ss.b3;
            x += c.bulkPi * (r1 * m2 * cf.x + r3 * cf.z);
            y += c.bulkPi * r2 * cf.y;
        }
    }
    x *= da.x;
    y *= da.x;
    if (kDiff) {
        const float r4 = m2 * T * T * ss.q1;
        const float r5 = (T * T * T / 3.0f) * ss.q2;
        const float dq = c.dsq * c.inv_kappa;
        x -= dq * c.pref_q * r4;
        y -= dq * r5;
    }
    return make_float2(c.unit_pref * x, c.unit_pref * y);
}

// negative -> 0 (FSSW::calculate_dN_dxtdy_for_one_particle_species,
// src/FSSW.cpp:707); NaN -> 0; +inf -> FLT_MAX so the cell CDF stays
// finite; -0 -> +0 so the bits order as the values
__device__ __forceinline__ float member_yield(const SpeciesDev& sp, float2 xy) {
    const float total = sp.degen * fmaf(static_cast<float>(sp.baryon), xy.y, xy.x);
    return __uint_as_float(__float_as_uint(fminf(fmaxf(total, 0.0f), 3.40282347e38f)) & 0x7FFFFFFFu);
}

// Yields of the species groups k0, k0 + kstep, ... in cell l (not dropped:
// u.dsigma >= 0).  A group's series runs for its first member and is reused
// by the next members while their chemical potential in this cell has the
// same bits (the same inputs, so the same sums); a member with another mu
// gets its own series.
template <bool kDiff>
__device__ __forceinline__ void cell_yields(const DevConfig& cfg, const CellArrays& cells,
                                            const SpeciesDev* s_sp, const int32_t* s_gst,
                                            const int32_t* s_mem, int n_groups, int k0, int kstep,
                                            int64_t n, int64_t l, float4 da, bool valid, bool live,
                                            uint32_t* s_max, uint32_t* __restrict__ ymax_row,
                                            float* __restrict__ yields) {
    CellYieldIn c;
    const int64_t lc = valid ? l : 0;   // lanes past the last cell read cell 0 and store nothing
    c.th = cells.th[lc];
    c.th2 = cells.th2[lc];
    c.cf = cells.coef[lc];
    const float4 th = c.th, th2 = c.th2, cf = c.cf;
    const float T = th.x;
    const double beta_d = 1.0 / static_cast<double>(T);
    const float b_hi = static_cast<float>(beta_d);
    const float b_lo = static_cast<float>(beta_d - static_cast<double>(b_hi));
    const bool warm = static_cast<double>(T) > 0.05;
    const int bulk_kind = cfg.bulk_kind;
    const bool with_bulk = cfg.include_bulk != 0;
    constexpr bool with_diff = kDiff;
    const bool kind_ce = (bulk_kind == 1 || bulk_kind == 21);
    const bool kind_14 = (bulk_kind == 11 || bulk_kind == 20);
    float bulkPi = 0.0f;
    if (with_bulk) bulkPi = (bulk_kind == 21 || bulk_kind == 20 || bulk_kind == 11 || bulk_kind == 0)
                                ? th2.w : th2.w / kHbarCf;
    float dsq = 0.0f, pref_q = 0.0f, inv_kappa = 0.0f;
    if (with_diff) {
        const float4 p2 = cells.pi2[lc];
        dsq = p2.y * da.y + p2.z * da.z + p2.w * da.w;
        pref_q = th2.z / (th2.x + th2.y);
        inv_kappa = 1.0f / cf.w;
    }
    // (1/hbarc^3) / (2 pi^2)
    const float unit_pref = (1.0f / (0.197327053f * 0.197327053f * 0.197327053f)) /
                            (2.0f * 9.8696044010893586f);

    c.T = T;
    c.b_hi = b_hi;
    c.b_lo = b_lo;
    c.warm = warm;
    c.with_bulk = with_bulk;
    c.kind_ce = kind_ce;
    c.kind_14 = kind_14;
    c.bulk_kind = bulk_kind;
    c.bulkPi = bulkPi;
    c.dsq = dsq;
    c.pref_q = pref_q;
    c.inv_kappa = inv_kappa;
    c.unit_pref = unit_pref;
    for (int j = k0; j < n_groups; j += kstep) {
        const int a = s_gst[j], b = s_gst[j + 1];
        float2 xy = make_float2(0.0f, 0.0f);
        uint32_t mu_bits = 0;
        for (int t = a; t < b; t++) {
            const int k = s_mem[t];
            const SpeciesDev sp = s_sp[k];
            float yv = 0.0f;
            if (live) {
                const float mu = species_mu(sp, th);
                if (t == a || __float_as_uint(mu) != mu_bits) {
                    xy = yield_coefs<kDiff>(c, sp, thermal_series<kDiff>(cfg, c, sp, mu), da);
                    mu_bits = __float_as_uint(mu);
                }
                yv = member_yield(sp, xy);
            }
            if (valid) yields[static_cast<int64_t>(k) * n + l] = yv;
            // the species' largest yield (its float bits: yields are >= +0,
            // so the unsigned order of the bits is the order of the values)
            const uint32_t m = __reduce_max_sync(0xffffffffu, __float_as_uint(yv));
            if ((threadIdx.x & 31) == 0 && m) {
                if (s_max) atomicMax(s_max + k, m);
                else atomicMax(ymax_row + k, m);
            }
        }
    }
}

// kDiff: include_deltaf_diffusion (a separate instantiation, so the common
// case carries none of the diffusion series' registers; it is held to 6
// blocks per SM, whose few spills cost less than the warps they add).  Besides the
// yields, the kernel raises ymax[b S + k] to the largest yield of species k
// on surface b (as float bits; ymax starts at 0): through a per-block
// maximum in shared memory when the block's cells lie on one surface, else
// lane by lane.
template <bool kDiff>
__global__ void __launch_bounds__(kYieldThreads, kDiff ? 4 : 6)
yields_kernel(DevConfig cfg, CellArrays cells, const SpeciesDev* __restrict__ species,
              float* __restrict__ yields, uint32_t* __restrict__ ymax) {
    extern __shared__ SpeciesDev s_sp[];
    __shared__ int s_b[2];
    const int nsp = cfg.n_species;
    const int G = cfg.n_ygroups;
    int32_t* s_gst = reinterpret_cast<int32_t*>(s_sp + nsp);
    int32_t* s_mem = s_gst + G + 1;
    uint32_t* s_max = reinterpret_cast<uint32_t*>(s_mem + nsp);
    const int64_t n = cfg.n_cells;
    const int64_t first = static_cast<int64_t>(blockIdx.x) * blockDim.x;
    for (int k = threadIdx.x; k < nsp; k += blockDim.x) {
        s_sp[k] = species[k];
        s_max[k] = 0u;
    }
    for (int k = threadIdx.x; k < G + 1 + nsp; k += blockDim.x) s_gst[k] = cfg.yorder[k];
    if (threadIdx.x < 2) {
        const int64_t lb = threadIdx.x == 0 ? first : min(first + blockDim.x, n) - 1;
        s_b[threadIdx.x] = surface_of(cfg.surf, cfg.n_surfaces, lb);
    }
    __syncthreads();
    const int64_t l = first + threadIdx.x;
    const bool valid = l < n;
    const bool one_surface = s_b[0] == s_b[1];
    const int b = one_surface ? s_b[0] : surface_of(cfg.surf, cfg.n_surfaces, valid ? l : n - 1);
    // blockIdx.y picks every gridDim.y-th species group: the groups come in
    // decreasing order of work, so interleaving keeps the rows' work equal,
    // and the grid has several waves of blocks
    const int k0 = blockIdx.y, kstep = gridDim.y;
    const float4 da = cells.da[valid ? l : 0];
    const bool live = valid && !(da.x < 0.0f);
    cell_yields<kDiff>(cfg, cells, s_sp, s_gst, s_mem, G, k0, kstep, n, l, da, valid, live,
                       one_surface ? s_max : nullptr, ymax + static_cast<int64_t>(b) * nsp,
                       yields);
    if (one_surface) {
        __syncthreads();
        for (int k = threadIdx.x; k < nsp; k += blockDim.x)
            if (s_max[k]) atomicMax(ymax + static_cast<int64_t>(s_b[0]) * nsp + k, s_max[k]);
    }
}

// ------------------------------------------------------------------------
// per-species fixed-point prefix sums over cells (cdf_quantize): tile sums,
// tile offsets and totals, tile scan with the guide-table scatter

constexpr int kScanThreads = 256;
constexpr int kScanPer = 8;
constexpr int kScanTile = kScanThreads * kScanPer;

__device__ __forceinline__ unsigned long long warp_incl_scan_u64(unsigned long long v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// exclusive block scan of one value per thread; returns the block total
__device__ unsigned long long block_excl_scan_u64(unsigned long long v, unsigned long long* s_warp,
                                                  unsigned long long* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned long long inc = warp_incl_scan_u64(v);
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        const unsigned long long w = lane < nw ? s_warp[lane] : 0ull;
        const unsigned long long wi = warp_incl_scan_u64(w);
        if (lane < nw) s_warp[lane] = wi - w;
        if (lane == nw - 1) s_warp[32] = wi;
    }
    __syncthreads();
    const unsigned long long out = s_warp[wid] + inc - v;
    *total = s_warp[32];
    __syncthreads();
    return out;
}

// Scan tiles are numbered over all rows (b, k) of the batch: surface b owns
// tiles [tile_base, tile_base + S nt) -- species k's row is its k-th run of
// nt tiles.  A block finds its surface by binary search over tile_base.
struct TileRef {
    const SurfSeg* sg;
    int b, k;
    int64_t tile;             // tile index inside the row
};

__device__ __forceinline__ TileRef tile_ref(const SurfSeg* __restrict__ surf, int n_surf, int S,
                                            int64_t t) {
    int lo = 0, hi = n_surf - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (surf[mid].tile_base <= t) lo = mid; else hi = mid - 1;
    }
    TileRef r;
    r.sg = surf + lo;
    r.b = lo;
    const int64_t local = t - r.sg->tile_base;
    r.k = static_cast<int>(local / r.sg->nt);
    r.tile = local - static_cast<int64_t>(r.k) * r.sg->nt;
    if (r.k >= S) r.k = S - 1;   // not reached: the grid has exactly the batch's tiles
    return r;
}

__global__ void __launch_bounds__(kScanThreads)
cdf_tile_sum_kernel(const float* __restrict__ yields, int64_t N, const SurfSeg* __restrict__ surf,
                    int n_surf, int S, const uint32_t* __restrict__ ymax,
                    unsigned long long* __restrict__ tile_sum) {
    __shared__ unsigned long long s_warp[kScanThreads / 32];
    const TileRef tr = tile_ref(surf, n_surf, S, blockIdx.x);
    const int64_t n = tr.sg->n;
    const int64_t t0 = tr.tile * kScanTile;
    const uint32_t* row =
        reinterpret_cast<const uint32_t*>(yields + static_cast<int64_t>(tr.k) * N + tr.sg->c0);
    const int base = cdf_quant_base(ymax[tr.b * S + tr.k], tr.sg->L);
    uint32_t v[kScanPer];
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
        const int64_t i = t0 + k * kScanThreads + threadIdx.x;
        v[k] = i < n ? __ldg(row + i) : 0u;
    }
    unsigned long long acc = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) acc += cdf_quantize(v[k], base);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
#pragma unroll
        for (int w = 0; w < kScanThreads / 32; w++) t += s_warp[w];
        tile_sum[blockIdx.x] = t;
    }
}

// one block per row (b, k): exclusive scan of the row's tile sums, the row
// total Q, the FP64 yield Q 2^-E, C[n] = Q and the guide sentinel
__global__ void __launch_bounds__(kScanThreads)
cdf_tile_offset_kernel(const SurfSeg* __restrict__ surf, int S,
                       const unsigned long long* __restrict__ tile_sum,
                       const uint32_t* __restrict__ ymax, unsigned long long* __restrict__ tile_off,
                       unsigned long long* __restrict__ qtot, double* __restrict__ totals,
                       unsigned long long* __restrict__ cdf, int32_t* __restrict__ guide) {
    __shared__ unsigned long long s_warp[33];
    const int r = blockIdx.x;
    const int b = r / S, k = r - b * S;
    const SurfSeg sg = surf[b];
    const int64_t first = sg.tile_base + static_cast<int64_t>(k) * sg.nt;
    unsigned long long carry = 0;
    for (int i0 = 0; i0 < sg.nt; i0 += kScanThreads) {
        const int i = i0 + threadIdx.x;
        const unsigned long long v = i < sg.nt ? tile_sum[first + i] : 0ull;
        unsigned long long tot;
        const unsigned long long ex = block_excl_scan_u64(v, s_warp, &tot);
        if (i < sg.nt) tile_off[first + i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        const int base = cdf_quant_base(ymax[r], sg.L);
        qtot[r] = carry;
        totals[r] = carry ? ldexp(static_cast<double>(carry), -(150 + base)) : 0.0;
        cdf[sg.cdf_base + static_cast<int64_t>(k) * (sg.n + 1) + sg.n] = carry;
        const int64_t G = int64_t(1) << sg.g;
        guide[sg.guide_base + static_cast<int64_t>(k) * (G + 1) + G] = static_cast<int32_t>(sg.n - 1);
    }
}

// f(j) = floor(j * Q / 2^g): the smallest v of guide bucket j (r >> (64 - g) == j)
__device__ __forceinline__ unsigned long long bucket_start(unsigned long long j, int g,
                                                           unsigned long long Q) {
    return __umul64hi(j << (64 - g), Q);
}

// Writes row (b, k) of the cell CDF, C[i] = sum of q over cells < i, and
// scatters the guide table (indexed search, Chen & Asau 1974): guide[j] is
// the cell whose interval [C[i], C[i+1]) holds f(j).  The intervals partition
// [0, Q), so every bucket j < 2^g gets exactly one writer; the cell of any v
// drawn in bucket j lies in [guide[j], guide[j+1]].
__global__ void __launch_bounds__(kScanThreads)
cdf_tile_scan_kernel(const float* __restrict__ yields, int64_t N, const SurfSeg* __restrict__ surf,
                     int n_surf, int S, const uint32_t* __restrict__ ymax,
                     const unsigned long long* __restrict__ tile_off,
                     const unsigned long long* __restrict__ qtot,
                     unsigned long long* __restrict__ cdf, int32_t* __restrict__ guide) {
    // padded tile buffers: element e of the tile sits at (e / 8) * 9 + e % 8;
    // s_in holds the FP32 yield bits, s_c the CDF values on the way out
    __shared__ uint32_t s_in[kScanThreads * (kScanPer + 1)];
    __shared__ unsigned long long s_c[kScanThreads * (kScanPer + 1)];
    __shared__ unsigned long long s_warp[33];
    const TileRef tr = tile_ref(surf, n_surf, S, blockIdx.x);
    const int64_t n = tr.sg->n;
    const int r = tr.b * S + tr.k;
    const int64_t t0 = tr.tile * kScanTile;
    const uint32_t* row =
        reinterpret_cast<const uint32_t*>(yields + static_cast<int64_t>(tr.k) * N + tr.sg->c0);
    unsigned long long* out = cdf + tr.sg->cdf_base + static_cast<int64_t>(tr.k) * (n + 1);
    const int g = tr.sg->g;
    const int64_t G = int64_t(1) << g;
    int32_t* gd = guide + tr.sg->guide_base + static_cast<int64_t>(tr.k) * (G + 1);
    const int base = cdf_quant_base(ymax[r], tr.sg->L);
    const unsigned long long Q = qtot[r];
    // coalesced load
    for (int k = 0; k < kScanPer; k++) {
        const int e = k * kScanThreads + threadIdx.x;
        const int64_t i = t0 + e;
        s_in[(e / kScanPer) * (kScanPer + 1) + e % kScanPer] = i < n ? row[i] : 0u;
    }
    __syncthreads();
    const uint32_t* mine = s_in + threadIdx.x * (kScanPer + 1);
    unsigned long long* mine_c = s_c + threadIdx.x * (kScanPer + 1);
    unsigned long long acc = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
        const unsigned long long q = cdf_quantize(mine[k], base);
        mine_c[k] = q;
        acc += q;
    }
    unsigned long long tot;
    const unsigned long long ex = block_excl_scan_u64(acc, s_warp, &tot);
    const unsigned long long start = tile_off[blockIdx.x] + ex;
    const int64_t e0 = t0 + static_cast<int64_t>(threadIdx.x) * kScanPer;
    // q -> exclusive prefix C, in place
    unsigned long long run = start;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
        const unsigned long long q = mine_c[k];
        mine_c[k] = run;
        run += q;
    }
    __syncthreads();
    // coalesced store of C[t0 .. t0 + tile)
    for (int k = 0; k < kScanPer; k++) {
        const int e = k * kScanThreads + threadIdx.x;
        const int64_t i = t0 + e;
        if (i < n) out[i] = s_c[(e / kScanPer) * (kScanPer + 1) + e % kScanPer];
    }
    if (Q == 0 || e0 >= n || run == start) return;
    // Guide scatter.  Bucket j starts at f(j) = floor(j Q / G) = j qd + floor(j qr / G)
    // with Q = qd G + qr; f is stepped exactly: f(j+1) = f(j) + qd + carry.
    // First bucket at or after this thread's first cell: a float estimate of
    // ceil(start G / Q), then exact steps.
    // (the top 24 significant bits of Q and start, converted exactly from
    // 32-bit integers: within a bucket of the answer for g <= 22)
    const int qsh = max(0, 40 - __clzll(static_cast<long long>(Q)));
    int64_t j = static_cast<int64_t>(
        static_cast<float>(static_cast<uint32_t>(start >> qsh)) *
        __fdividef(static_cast<float>(G), static_cast<float>(static_cast<uint32_t>(Q >> qsh))));
    j = j < 0 ? 0 : (j > G ? G : j);
    while (j > 0 && bucket_start(static_cast<unsigned long long>(j - 1), g, Q) >= start) --j;
    while (j < G && bucket_start(static_cast<unsigned long long>(j), g, Q) < start) ++j;
    const unsigned long long qd = Q >> g, qr = Q & static_cast<unsigned long long>(G - 1);
    unsigned long long rem = (static_cast<unsigned long long>(j) * qr) & static_cast<unsigned long long>(G - 1);
    unsigned long long f = j < G ? bucket_start(static_cast<unsigned long long>(j), g, Q) : Q;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
        const unsigned long long hi = (k + 1 < kScanPer) ? mine_c[k + 1] : run;
        while (j < G && f < hi) {
            gd[j] = static_cast<int32_t>(e0 + k);
            ++j;
            rem += qr;
            f += qd + (rem >> g);
            rem &= static_cast<unsigned long long>(G - 1);
        }
    }
}

}  // namespace

// ------------------------------------------------------------------------
// launch wrappers

cudaError_t launch_yields(const DevConfig& cfg, const CellArrays& cells, const SpeciesDev* sp,
                          float* yields, uint32_t* ymax, cudaStream_t stream) {
    cudaError_t e0 = cudaMemsetAsync(
        ymax, 0, sizeof(uint32_t) * static_cast<size_t>(cfg.n_surfaces) * cfg.n_species, stream);
    if (e0 != cudaSuccess) return e0;
    if (cfg.n_cells <= 0) return cudaSuccess;
    const unsigned blocks = static_cast<unsigned>((cfg.n_cells + kYieldThreads - 1) / kYieldThreads);
    // species, group starts and members, per-block species maxima
    const size_t smem = sizeof(SpeciesDev) * static_cast<size_t>(cfg.n_species) +
                        sizeof(int32_t) * static_cast<size_t>(cfg.n_ygroups + 1 + 2 * cfg.n_species);
    auto kernel = cfg.include_diff ? yields_kernel<true> : yields_kernel<false>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    const int want = cfg.yield_groups > 0 ? cfg.yield_groups : kYieldGroups;
    const unsigned groups = static_cast<unsigned>(std::max(1, std::min(want, cfg.n_ygroups)));
    kernel<<<dim3(blocks, groups), kYieldThreads, smem, stream>>>(cfg, cells, sp, yields, ymax);
    return cudaGetLastError();
}

int cdf_num_tiles(int64_t n) { return static_cast<int>((n + kScanTile - 1) / kScanTile); }

cudaError_t launch_cdf_head(const float* yields, int64_t N, const SurfSeg* surf, int n_surf,
                            int64_t n_tiles, int S, uint32_t* ymax, unsigned long long* tile_sum,
                            unsigned long long* tile_off, unsigned long long* qtot, double* totals,
                            unsigned long long* cdf, int32_t* guide, cudaStream_t stream) {
    if (n_tiles <= 0 || S <= 0 || n_surf <= 0) return cudaSuccess;
    const int rows = n_surf * S;
    const unsigned grid = static_cast<unsigned>(n_tiles);
    cdf_tile_sum_kernel<<<grid, kScanThreads, 0, stream>>>(yields, N, surf, n_surf, S, ymax,
                                                          tile_sum);
    cdf_tile_offset_kernel<<<rows, kScanThreads, 0, stream>>>(surf, S, tile_sum, ymax, tile_off,
                                                             qtot, totals, cdf, guide);
    return cudaGetLastError();
}

cudaError_t launch_cdf_scan(const float* yields, int64_t N, const SurfSeg* surf, int n_surf,
                            int64_t n_tiles, int S, const uint32_t* ymax, const unsigned long long* tile_off,
                            const unsigned long long* qtot, unsigned long long* cdf, int32_t* guide,
                            cudaStream_t stream) {
    if (n_tiles <= 0 || S <= 0 || n_surf <= 0) return cudaSuccess;
    const unsigned grid = static_cast<unsigned>(n_tiles);
    cdf_tile_scan_kernel<<<grid, kScanThreads, 0, stream>>>(yields, N, surf, n_surf, S, ymax,
                                                           tile_off, qtot, cdf, guide);
    return cudaGetLastError();
}

cudaError_t launch_cdf(const float* yields, int64_t N, const SurfSeg* surf, int n_surf,
                       int64_t n_tiles, int S, uint32_t* ymax, unsigned long long* tile_sum,
                       unsigned long long* tile_off, unsigned long long* qtot, double* totals,
                       unsigned long long* cdf, int32_t* guide, cudaStream_t stream) {
    const cudaError_t e = launch_cdf_head(yields, N, surf, n_surf, n_tiles, S, ymax, tile_sum, tile_off,
                                          qtot, totals, cdf, guide, stream);
    if (e != cudaSuccess) return e;
    return launch_cdf_scan(yields, N, surf, n_surf, n_tiles, S, ymax, tile_off, qtot, cdf, guide, stream);
}

}  // namespace iss
