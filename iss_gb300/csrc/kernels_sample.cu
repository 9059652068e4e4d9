// Sampling kernels:
//   counts_kernel     FSSW::determine_number_to_sample (src/FSSW.cpp:250-309), one
//                     draw per (event, species) from the Philox stream
//                     {iteration, 0, event, species | TAG_COUNT << 16}
//   offsets scan      exclusive int64 prefix sum of the counts: each
//                     (event, species) segment gets its output slots, events in
//                     order, species in mass order inside an event (the order of
//                     src/FSSW.cpp:920-1049)
//   sampler_kernel    per hadron: cell draw on the species' FP64 CDF
//                     (RandomVariable1DArray::rand, src/RandomVariable1DArray.cpp:67-70),
//                     momentum by rejection in the local rest frame with the
//                     Cooper-Frye / delta-f weight (src/FSSW.cpp:1852-1966),
//                     boost to the lab and the hadron record
//                     (src/FSSW.cpp:1969-2010).
//
// The |p| proposal is an exact Gamma mixture: with K = (E - m)/T and
// m~ = m/T the density (E^2 - m^2/2) exp(-(E - mu)/T) is proportional to
// (K^2 + 2 m~ K + m~^2/2) exp(-K), a mixture of Gamma(3), Gamma(2) and
// Gamma(1) with weights 2, 2 m~ and m~^2/2.  The direction is proposed from
// the Cooper-Frye flux factor clamp01(p.dsigma / (p0 dsigma_fac)) of
// src/FSSW.cpp:1939-1941 itself: with dsigma_mu = (d0, D n) in the rest frame
// the factor is linear in cos(angle to n), so cos is drawn from that linear
// density (cut at its zero for spacelike cells) by inverse CDF, and the part of
// the flux weight that depends on |p| is left to the acceptance.  The
// quantum-statistics factor f/exp(-(E-mu)/T), the pE/(E^2 - m^2/2) factor of
// src/MomentumSamplerBase.cpp:45-56, that flux remainder and the delta-f factor
// clamp01((1 + delta f)/2) of src/FSSW.cpp:1942 are applied as one acceptance
// probability, so the accepted density is the reference's p^2 f(E) x accept.  The support is cut at the end of the reference's
// momentum table for the selected sampler (src/MomentumSamplerShell.cpp:24-48).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "device_common.cuh"
#include "kernels.h"
#include "learned_record.cuh"

namespace iss {

namespace {

constexpr float kTwoOverE10 = 0.0735758882342885f;   // 2 / (10 e)

__device__ __forceinline__ uint4 block(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                       uint32_t k0, uint32_t k1) {
    return philox4x32_10(make_uint4(c0, c1, c2, c3), k0, k1);
}

// ------------------------------------------------------------------------
// counts

// Poisson draws: inversion for mu < 12, PTRS (Hoermann 1993) above.  The
// FP64 expressions use explicitly rounded operations (__dmul_rn, __dadd_rn),
// so no multiply-add is contracted and the CPU replay gets the same bits.
struct PoissonC {
    double mu, emu;                 // mu, exp(-mu)          (inversion)
    double b, a, inv_alpha, vr;     // PTRS constants
    double log_mu, log_ia;          // log(mu), log(inv_alpha)
};
static_assert(sizeof(PoissonC) == kPoissonConsts * sizeof(double), "PoissonC layout");

// Inversion CDF of one species, cdf[0..len) as the inversion loop forms it,
// stopped where adding the next term no longer changes it (then every later
// term is smaller still); len = 0 when kInvTable entries do not reach that.
// Each entry is held as floor(cdf 2^53): the draw's uniform is an integer
// U times 2^-53 (u53), and u > cdf exactly when U > floor(cdf 2^53), so the
// search compares 64-bit integers (ALU) instead of doubles (FP64 pipe) and
// finds the same k.
struct PoissonInv {
    unsigned long long icdf[kInvTable];
    int len;
};
static_assert(sizeof(PoissonInv) == (kInvTable + 1) * sizeof(double), "PoissonInv layout");

__device__ __forceinline__ unsigned long long floor_2p53(double x) {
    // x in [0, 1]: x 2^53 is exact and below 2^53 + 1, truncation is floor
    return static_cast<unsigned long long>(x * 9007199254740992.0);
}

__device__ PoissonC poisson_consts(double mu) {
    PoissonC c{};
    c.mu = mu;
    if (mu < 12.0) {
        c.emu = exp(-mu);
        return c;
    }
    const double smu = sqrt(mu);
    c.b = __dadd_rn(0.931, __dmul_rn(2.53, smu));
    c.a = __dadd_rn(-0.059, __dmul_rn(0.02483, c.b));
    c.inv_alpha = __dadd_rn(1.1239, 1.1328 / __dadd_rn(c.b, -3.4));
    c.vr = __dadd_rn(0.9277, -(3.6224 / __dadd_rn(c.b, -2.0)));
    c.log_mu = log(mu);
    c.log_ia = log(c.inv_alpha);
    return c;
}

// log(k!): the table for k < kLogFactLen, else the Stirling series of
// lgamma(n), n = k + 1, to the n^-5 term (truncation below 1e-20 relative)
__device__ __forceinline__ double log_factorial(const double* __restrict__ table, double kd) {
    if (kd < static_cast<double>(kLogFactLen)) return table[static_cast<int>(kd)];
    const double n = __dadd_rn(kd, 1.0);
    const double r = 1.0 / n, r2 = __dmul_rn(r, r);
    const double t = __dadd_rn(1.0 / 12.0,
                               -__dmul_rn(r2, __dadd_rn(1.0 / 360.0, -__dmul_rn(r2, 1.0 / 1260.0))));
    return __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(__dadd_rn(n, -0.5), log(n)), -n),
                               0.91893853320467274178),
                     __dmul_rn(r, t));
}

__device__ void poisson_inv_table(const PoissonC& c, PoissonInv& t) {
    t.len = 0;
    if (!(c.mu < 12.0)) return;
    double p = c.emu, cdf = p;
    t.icdf[0] = floor_2p53(cdf);
    for (int k = 1; k < kInvTable; k++) {
        p = __dmul_rn(p, c.mu / static_cast<double>(k));
        const double next = __dadd_rn(cdf, p);
        if (next == cdf && static_cast<double>(k) > c.mu) {
            t.len = k;
            return;
        }
        cdf = next;
        t.icdf[k] = floor_2p53(cdf);
    }
}

__device__ int64_t poisson_draw(uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t iter0,
                                const PoissonC& c, const double* __restrict__ logfact,
                                const PoissonInv* __restrict__ inv = nullptr) {
    const double mu = c.mu;
    if (mu < 12.0) {
        const uint4 w = block(iter0, 0u, c2, c3, k0, k1);
        if (inv && inv->len > 0) {
            // first k with u <= cdf[k], u = U 2^-53; past the saturated end
            // the loop below would run to its cap
            const unsigned long long U = (static_cast<unsigned long long>(w.x >> 5) << 26) |
                                         static_cast<unsigned long long>(w.y >> 6);
            int lo = 0, hi = inv->len;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (U > inv->icdf[mid]) lo = mid + 1; else hi = mid;
            }
            return lo < inv->len ? lo : 1000;
        }
        const double u = u53(w.x, w.y);
        double p = c.emu;
        double cdf = p;
        int64_t k = 0;
        while (u > cdf && k < 1000) {
            k++;
            p = __dmul_rn(p, mu / static_cast<double>(k));
            cdf = __dadd_rn(cdf, p);
        }
        return k;
    }
    for (uint32_t it = 0; it < 10000u; it++) {
        const uint4 w = block(iter0 + it, 0u, c2, c3, k0, k1);
        const double U = __dadd_rn(u53(w.x, w.y), -0.5);
        const double V = u53(w.z, w.w);
        const double us = __dadd_rn(0.5, -fabs(U));
        const double kd = floor(__dadd_rn(
            __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(2.0, c.a) / us, c.b), U), mu), 0.43));
        if (us >= 0.07 && V <= c.vr) return static_cast<int64_t>(kd);
        if (kd < 0.0 || (us < 0.013 && V > us)) continue;
        const double lhs =
            __dadd_rn(__dadd_rn(log(V), c.log_ia), -log(__dadd_rn(c.a / __dmul_rn(us, us), c.b)));
        const double rhs =
            __dadd_rn(__dadd_rn(-mu, __dmul_rn(kd, c.log_mu)), -log_factorial(logfact, kd));
        if (lhs <= rhs) return static_cast<int64_t>(kd);
    }
    return -1;
}

__device__ double gamma_draw(uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t iter0,
                             double shape) {
    double boost = 1.0;
    if (shape < 1.0) {
        const uint4 w = block(iter0, 0u, c2, c3, k0, k1);
        boost = pow(static_cast<double>(u01f_pos(w.x)), 1.0 / shape);
        shape += 1.0;
        iter0 += 1;
    }
    const double d = shape - 1.0 / 3.0;
    const double cc = 1.0 / sqrt(9.0 * d);
    for (uint32_t it = 0; it < 10000u; it++) {
        const uint4 w = block(iter0 + it, 0u, c2, c3, k0, k1);
        const double r = sqrt(-2.0 * log(static_cast<double>(u01f_pos(w.x))));
        const double x = r * cos(2.0 * 3.14159265358979323846 * static_cast<double>(u01f(w.y)));
        double v = 1.0 + cc * x;
        if (v <= 0.0) continue;
        v = v * v * v;
        const double u = u53(w.z, w.w);
        if (u < 1.0 - 0.0331 * x * x * x * x) return boost * d * v;
        if (log(u) < 0.5 * x * x + d * (1.0 - v + log(v))) return boost * d * v;
    }
    return -1.0;
}

// a work item is cfg.item_size consecutive draws of one (event, species)
// segment; the cell assignment takes them 64 at a time (two per lane)
constexpr int kAssignSub = 64;
constexpr float kTwoPiF = 6.2831853071795865f;
// guide buckets spanning at most this many cells past their first are
// resolved with one batch of CDF reads (cell_assign_kernel)
constexpr int kAssignSpan = 3;

// Work items are ordered by event chunk (cfg.chunk_events consecutive events),
// then species, then event: warps that run at the same time mostly sample one
// species, whose cell CDF and guide table stay in L2, and the items of one
// chunk are contiguous, so a chunk can be sampled (and its records copied
// out) before the next.  The output slots stay event-major.
__device__ __forceinline__ int64_t item_index(const DevConfig& cfg, int e, int s) {
    const int c = e / cfg.chunk_events;
    const int e0 = c * cfg.chunk_events;
    const int ne = min(cfg.chunk_events, cfg.n_events - e0);
    return static_cast<int64_t>(e0) * cfg.n_species + static_cast<int64_t>(s) * ne + (e - e0);
}

// local_charge_conservation: every hadron of a positively charged species is
// followed in its event by a partner of the same mass and opposite quantum
// numbers sampled in the same cell; negatively charged species are not
// sampled on their own (src/FSSW.cpp:931-938, 1035-1048).  A segment of a
// positive species then holds two records per draw.
__device__ __forceinline__ int records_per_draw(const DevConfig& cfg, const SpeciesDev& sp) {
    return (cfg.lcc && sp.charge > 0) ? 2 : 1;
}

__device__ __forceinline__ void item_decode(const DevConfig& cfg, int q, int& e, int& s) {
    const int per = cfg.chunk_events * cfg.n_species;
    const int c = q / per;
    const int e0 = c * cfg.chunk_events;
    const int ne = min(cfg.chunk_events, cfg.n_events - e0);
    const int r = q - c * per;
    s = r / ne;
    e = e0 + (r - s * ne);
}

// per-species Poisson constants of the model-30 draws (same mu in every event)
__global__ void count_consts_kernel(DevConfig cfg, const double* __restrict__ totals,
                                    PoissonC* __restrict__ pois, PoissonInv* __restrict__ inv) {
    // one thread per (surface, species) row
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= cfg.n_surfaces * cfg.n_species) return;
    const double dN = __dmul_rn(totals[s], cfg.ymult);
    const PoissonC c = poisson_consts(dN);
    pois[s] = c;
    poisson_inv_table(c, inv[s]);
}

__global__ void counts_kernel(DevConfig cfg_in, const SpeciesDev* __restrict__ species,
                              const double* __restrict__ totals,
                              const PoissonC* __restrict__ pois,
                              const PoissonInv* __restrict__ inv, int32_t* __restrict__ counts,
                              int32_t* __restrict__ items, int* __restrict__ error) {
    const DevConfig cfg = with_run_keys(cfg_in);
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t total = static_cast<int64_t>(cfg.n_events) * cfg.n_species;
    if (idx >= total) return;
    // species-major threads: a warp draws one species in consecutive events,
    // so its lanes take the same branch (inversion table or PTRS) and read
    // the same constants; every draw is keyed by (event, species)
    const int s = static_cast<int>(idx / cfg.n_events);
    const int e = static_cast<int>(idx % cfg.n_events);
    const int64_t seg = static_cast<int64_t>(e) * cfg.n_species + s;
    const uint32_t c2 = cfg.event_offset + static_cast<uint32_t>(e);
    const uint32_t c3 = static_cast<uint32_t>(s) | (kTagCount << 16);
    const int row = cfg.ev_surf[e] * cfg.n_species + s;    // (surface, species)
    const double dN = __dmul_rn(totals[row], cfg.ymult);
    const int64_t dN_int = static_cast<int64_t>(dN);
    const double frac = __dadd_rn(dN, -static_cast<double>(dN_int));
    const double para1 = cfg.sampling_para1;
    int64_t nsamp = 0;
    const SpeciesDev sp = species[s];
    if (cfg.lcc && sp.charge < 0) {
        nsamp = 0;   // sampled as partners of the positive species
    } else if (dN < 0) {
        atomicCAS(error, 0, 2);
    } else if (cfg.sampling_model == 1) {
        const uint4 w = block(0u, 0u, c2, c3, cfg.key0, cfg.key1);
        nsamp = dN_int + (u53(w.x, w.y) < frac ? 1 : 0);
    } else if (cfg.sampling_model == 10 || cfg.sampling_model == 20) {
        const double kk = (cfg.sampling_model == 10) ? __dmul_rn(para1, frac) : __dmul_rn(para1, dN);
        const double p = 1.0 / __dadd_rn(1.0, para1);
        if (kk < 1e-15) {
            nsamp = dN_int;
        } else {
            const double g = gamma_draw(c2, c3, cfg.key0, cfg.key1, 0u, kk);
            const PoissonC pc = poisson_consts(__dmul_rn(g, __dadd_rn(1.0, -p)) / p);
            const int64_t nb = poisson_draw(c2, c3, cfg.key0, cfg.key1, 1u << 20, pc, cfg.tab.logfact);
            nsamp = (cfg.sampling_model == 10) ? dN_int + nb : nb;
            if (g < 0.0 || nb < 0) atomicCAS(error, 0, 3);
        }
    } else {
        nsamp = (dN < 1e-15) ? 0
                             : poisson_draw(c2, c3, cfg.key0, cfg.key1, 0u, pois[row],
                                            cfg.tab.logfact, inv + row);
        if (nsamp < 0) atomicCAS(error, 0, 3);
    }
    const int32_t c = static_cast<int32_t>(nsamp < 0 ? 0 : nsamp);
    counts[seg] = c * records_per_draw(cfg, sp);       // records of the segment
    items[item_index(cfg, e, s)] = (c + cfg.item_size - 1) / cfg.item_size;
}

// item -> segment map: item_seg[item_off[q] + k] = q for k < items[q], q the
// work-item order index of the segment (item_index)
__global__ void item_map_kernel(const int32_t* __restrict__ items, const int64_t* __restrict__ item_off,
                                int64_t nseg, int32_t* __restrict__ item_seg,
                                const int64_t* __restrict__ limits) {
    const int64_t seg = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (seg >= nseg) return;
    // graph replays: nothing is written when the buffers are too small
    if (limits && limits[1] != 0) return;
    const int64_t b = item_off[seg];
    const int32_t k = items[seg];
    for (int32_t j = 0; j < k; j++) item_seg[b + j] = static_cast<int32_t>(seg);
}

// graph replays: the work-item count of this call (limits[0]) and whether the
// call fits the buffers the graph was captured with (limits[1] = 1: it does
// not; then nothing is sampled and the host reruns the call eagerly)
__global__ void graph_limits_kernel(const int64_t* __restrict__ offsets,
                                    const int64_t* __restrict__ item_off, int64_t nseg,
                                    int64_t cap_units, int64_t cap_items, int64_t* __restrict__ limits) {
    const int64_t units = offsets[nseg], n_items = item_off[nseg];
    const bool fits = units <= cap_units && n_items <= cap_items;
    limits[0] = fits ? n_items : 0;
    limits[1] = fits ? 0 : 1;
}

// ------------------------------------------------------------------------
// exclusive int64 scan of the counts

constexpr int kOffThreads = 256;
constexpr int kOffPer = 16;
constexpr int kOffTile = kOffThreads * kOffPer;

__device__ __forceinline__ long long warp_incl_scan_ll(long long v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

__device__ long long block_excl_scan_ll(long long v, long long* s_warp, long long* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const long long inc = warp_incl_scan_ll(v);
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        const long long w = lane < nw ? s_warp[lane] : 0;
        const long long wi = warp_incl_scan_ll(w);
        if (lane < nw) s_warp[lane] = wi - w;
        if (lane == nw - 1) s_warp[32] = wi;
    }
    __syncthreads();
    const long long out = s_warp[wid] + inc - v;
    *total = s_warp[32];
    __syncthreads();
    return out;
}

__global__ void __launch_bounds__(kOffThreads)
off_tile_sum_kernel(const int32_t* __restrict__ counts, int64_t n, int64_t* __restrict__ tile_sum) {
    __shared__ long long s_warp[33];
    const int64_t t0 = static_cast<int64_t>(blockIdx.x) * kOffTile;
    long long acc = 0;
    for (int k = 0; k < kOffPer; k++) {
        const int64_t i = t0 + k * kOffThreads + threadIdx.x;
        if (i < n) acc += counts[i];
    }
    long long tot;
    block_excl_scan_ll(acc, s_warp, &tot);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kOffThreads)
off_tile_offset_kernel(int64_t* __restrict__ tile_sum, int n_tiles, int64_t* __restrict__ offsets,
                       int64_t n) {
    __shared__ long long s_warp[33];
    long long carry = 0;
    for (int b = 0; b < n_tiles; b += kOffThreads) {
        const int i = b + threadIdx.x;
        const long long v = i < n_tiles ? tile_sum[i] : 0;
        long long tot;
        const long long ex = block_excl_scan_ll(v, s_warp, &tot);
        if (i < n_tiles) tile_sum[i] = carry + ex;   // in place: now tile offsets
        carry += tot;
    }
    if (threadIdx.x == 0) offsets[n] = carry;
}

__global__ void __launch_bounds__(kOffThreads)
off_tile_scan_kernel(const int32_t* __restrict__ counts, int64_t n,
                     const int64_t* __restrict__ tile_off, int64_t* __restrict__ offsets) {
    __shared__ int32_t s_in[kOffThreads * (kOffPer + 1)];
    __shared__ long long s_warp[33];
    const int64_t t0 = static_cast<int64_t>(blockIdx.x) * kOffTile;
    for (int k = 0; k < kOffPer; k++) {
        const int e = k * kOffThreads + threadIdx.x;
        const int64_t i = t0 + e;
        s_in[(e / kOffPer) * (kOffPer + 1) + e % kOffPer] = i < n ? counts[i] : 0;
    }
    __syncthreads();
    const int32_t* mine = s_in + threadIdx.x * (kOffPer + 1);
    long long acc = 0;
#pragma unroll
    for (int k = 0; k < kOffPer; k++) acc += mine[k];
    long long tot;
    long long run = tile_off[blockIdx.x] + block_excl_scan_ll(acc, s_warp, &tot);
    const int64_t e0 = t0 + static_cast<int64_t>(threadIdx.x) * kOffPer;
#pragma unroll
    for (int k = 0; k < kOffPer; k++) {
        if (e0 + k < n) offsets[e0 + k] = run;
        run += mine[k];
    }
}

// ------------------------------------------------------------------------
// sampler

struct Prop {
    float T, m, a, mt, Kmax, W, w32, w3, qa;
    // three-term Bose proposal (prop_bose2): W1 the weight of the e^-E~
    // term, W12 that of the first two (W adds e^-3E~), r2 = 4 e^a; W1 = W12 =
    // W for a one-term proposal
    float W1, W12, r2;
    float mut, cpoly, rmax;
    int compat, sign;
    // flux geometry in the LRF: dsigma_mu = (d0, D n); e1 _|_ n is rebuilt
    // from n and its norm einv by e1() (three registers fewer per lane)
    float d0, D, nx, ny, nz, einv;
    float pxx, pxy, pxz, pyy, pyz, shear_c;
    float bi0, b0, b1, b2;
    float qx, qy, qz, pq, Bq;
};

// e1 = normalised (t x n), t the coordinate axis least parallel to n: z when
// |n_z| < 0.9, else x
__device__ __forceinline__ void prop_e1(const Prop& p, float& ex, float& ey, float& ez) {
    if (fabsf(p.nz) < 0.9f) {
        ex = -p.ny * p.einv;
        ey = p.nx * p.einv;
        ez = 0.0f;
    } else {
        ex = 0.0f;
        ey = -p.nz * p.einv;
        ez = p.ny * p.einv;
    }
}

struct Unit {
    int64_t slot;
    uint32_t i, eg;
    int s;
    int cell;
    int redraw;
    int tries_cell;
    uint32_t t;                // tries made so far (proposal counter)
    int mult;                  // records per draw (2: local charge conservation pair)
    int phase;                 // 1: sampling the partner of a pair
    const float* lp;           // learned sampler: the pair's mixture record (null: plain)
};

// Cell draw from 64 random bits r on the fixed-point CDF row C[0..n]
// (cdf_quantize): v = floor(r * Q / 2^64), and the cell is the i with
// C[i] <= v < C[i+1] -- the reference's binarySearch (src/arsenal.cpp:644-678)
// on integer sums.  The guide bucket j = r >> (64 - g) brackets the cell by
// guide[j] <= i <= guide[j+1]; when both agree no CDF entry is read.
__device__ __forceinline__ int cell_search(const unsigned long long* __restrict__ row, int64_t n,
                                           const int32_t* __restrict__ gd, int g,
                                           unsigned long long Q, unsigned long long r) {
    const unsigned long long v = __umul64hi(r, Q);
    const unsigned j = static_cast<unsigned>(r >> (64 - g));
    const int2 b = make_int2(__ldg(gd + j), __ldg(gd + j + 1));
    const int last = static_cast<int>(n - 1);
    int lo = min(max(b.x, 0), last), hi = min(max(b.y, lo), last);
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(row + mid) <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// returns false when m/T - mu/T is outside the reference's momentum tables.
// The lean instantiations (no compat-fermion correction, with or without
// diffusion, kDiff) take the cell-only constants precomputed by the prologue
// (CellArrays::srec); the rest is setup_prop's own arithmetic
template <bool kDiff>
__device__ bool setup_prop_lean(const DevConfig& cfg, const CellArrays& cells, const SpeciesDev& sp,
                                int l, Prop& p) {
    const float4* sr = cells.srec + 8 * static_cast<int64_t>(l);
    const float4 fr = __ldg(sr + 2);   // d0, D, einv, T
    const float4 nb = __ldg(sr + 3);   // n, 1/T
    const float4 mu4 = __ldg(sr + 4);
    const float4 sh1 = __ldg(sr + 5);
    const float4 sh2 = __ldg(sr + 6);
    const float T = fr.w;
    const float beta = nb.w;
    const float m = sp.m_hi + sp.m_lo;
    const float mu_raw = static_cast<float>(sp.baryon) * mu4.x + static_cast<float>(sp.strange) * mu4.y +
                         static_cast<float>(sp.charge) * mu4.z;
    const float mu = fminf(m, mu_raw);
    p.T = T;
    p.m = m;
    p.sign = sp.sign;
    p.mt = m * beta;
    p.mut = mu * beta;
    p.a = (m - mu) * beta;
    const int sampler = p.a < 30.0f ? 0 : (p.a < 50.0f ? 1 : 2);
    float e0, de;
    int npts;
    if (p.sign == -1) {
        e0 = (sampler == 0 ? 0.05f : (sampler == 1 ? 30.0f : 50.0f)) + 0.05f;
        de = 0.05f;
        npts = 1001;
    } else {
        e0 = (sampler == 0 ? 0.0f : (sampler == 1 ? 30.0f : 50.0f));
        de = 0.02f;
        npts = 2001;
    }
    const int idx_min = static_cast<int>((p.a - e0) / de);
    if (idx_min < 0 || idx_min >= npts - 1) return false;
    p.Kmax = e0 + (npts - 1) * de - p.a;
    p.w3 = 2.0f;
    p.w32 = 2.0f + 2.0f * p.mt;
    p.W = p.w32 + 0.5f * p.mt * p.mt;
    p.qa = p.a > 0.05f ? 1.0f - __expf(-p.a) : -expm1f(-p.a);   // as a_q's denominator in the try
    p.compat = 0;
    p.cpoly = p.mut * p.mut - 0.5f * p.mt * p.mt;
    p.rmax = 1.0f;
    p.d0 = fr.x;
    p.D = fr.y;
    p.einv = fr.z;
    p.nx = nb.x;
    p.ny = nb.y;
    p.nz = nb.z;
    // shear tensor already times its prefactor
    p.pxx = sh1.x;
    p.pxy = sh1.y;
    p.pxz = sh1.z;
    p.pyy = sh1.w;
    p.pyz = sh2.x;
    p.shear_c = 1.0f;
    p.bi0 = p.b0 = p.b1 = p.b2 = 0.0f;
    if (cfg.include_bulk) {
        if (cfg.bulk_kind == 11) {
            p.b0 = sh2.y * (m * m);
            p.b1 = sh2.z * static_cast<float>(sp.baryon);
            p.b2 = sh2.w;
        } else if (cfg.bulk_kind == 21 || cfg.bulk_kind == 1) {
            p.bi0 = __ldg(sr + 7).x * (m * m);
            p.b1 = sh2.z;
        }
    }
    p.qx = p.qy = p.qz = p.pq = p.Bq = 0.0f;
    if (kDiff && cfg.include_diff) {
        const float4 dq = __ldg(sr + 7);   // q / kappa_B in its yzw
        p.qx = dq.y;
        p.qy = dq.z;
        p.qz = dq.w;
        p.pq = mu4.w;                      // n_B / (e + P)
        p.Bq = static_cast<float>(sp.baryon);
    }
    return true;
}

// kMode 0: every configuration, from the cell record; 1: lean (no diffusion,
// no compat-fermion factor), from the prologue's lean record; 2: the same
// with diffusion
template <int kMode = 0>
__device__ bool setup_prop(const DevConfig& cfg, const CellArrays& cells, const SpeciesDev& sp,
                           int l, Prop& p) {
    if (kMode != 0) return setup_prop_lean<kMode == 2>(cfg, cells, sp, l, p);
    constexpr bool kLean = false;
    const float4* rec = cells.rec + 8 * static_cast<int64_t>(l);
    const float4 da = __ldg(rec + 1);
    const float4 th = __ldg(rec + 3);
    const float4 th2 = __ldg(rec + 4);
    const float4 pi1 = __ldg(rec + 5);
    const float4 pi2 = __ldg(rec + 6);
    const float4 cf = __ldg(rec + 7);
    const float T = th.x;
    const float beta = 1.0f / T;
    const float m = sp.m_hi + sp.m_lo;
    const float mu_raw = static_cast<float>(sp.baryon) * th.y + static_cast<float>(sp.strange) * th.z +
                         static_cast<float>(sp.charge) * th.w;
    const float mu = fminf(m, mu_raw);
    p.T = T;
    p.m = m;
    p.sign = sp.sign;
    p.mt = m * beta;
    p.mut = mu * beta;
    p.a = (m - mu) * beta;
    const int sampler = p.a < 30.0f ? 0 : (p.a < 50.0f ? 1 : 2);
    float e0, de;
    int npts;
    if (p.sign == -1) {
        e0 = (sampler == 0 ? 0.05f : (sampler == 1 ? 30.0f : 50.0f)) + 0.05f;
        de = 0.05f;
        npts = 1001;
    } else {
        e0 = (sampler == 0 ? 0.0f : (sampler == 1 ? 30.0f : 50.0f));
        de = 0.02f;
        npts = 2001;
    }
    const int idx_min = static_cast<int>((p.a - e0) / de);
    if (idx_min < 0 || idx_min >= npts - 1) return false;
    p.Kmax = e0 + (npts - 1) * de - p.a;
    p.w3 = 2.0f;
    p.w32 = 2.0f + 2.0f * p.mt;
    p.W = p.w32 + 0.5f * p.mt * p.mt;
    p.qa = -expm1f(-p.a);
    p.compat = (!kLean && cfg.compat_fermion && sampler == 0) ? 1 : 0;
    p.cpoly = p.mut * p.mut - 0.5f * p.mt * p.mt;
    p.rmax = 1.0f;
    if (p.compat) {
        const float amu = fabsf(p.mut);
        if (p.sign == -1) {
            p.rmax = 1.0f + (p.mut < 0.0f ? 2.0f * amu * kTwoOverE10 / (p.mt * p.mt) : 0.0f);
        } else {
            const float r = 1.0f - p.mut / p.mt;
            const float C = fmaxf(1.0f, 2.0f * r * r);
            const float aa = fmaxf(p.a, 0.1f);
            const float x2 = (p.a >= 0.1f) ? aa * expf(-10.0f * aa) : 0.5f * kTwoOverE10;
            p.rmax = 1.0f + C * 2.0f / expm1f(fmaxf(p.a, 1e-12f)) + 8.0f * amu * x2 / (p.mt * p.mt);
        }
        // the bound is attained (fermions at threshold, bosons as E -> inf):
        // a relative margin keeps rounding from crossing it
        p.rmax *= 1.0f + 1e-5f;
    }
    // Cooper-Frye flux geometry: p.dsigma = p0 d0 + |p| D cos(alpha), alpha
    // measured from n; directions are proposed from this flux exactly
    p.d0 = fabsf(da.x);
    p.D = sqrtf(da.y * da.y + da.z * da.z + da.w * da.w);
    if (p.D > 1e-30f) {
        const float inv = 1.0f / p.D;
        p.nx = da.y * inv;
        p.ny = da.z * inv;
        p.nz = da.w * inv;
    } else {
        p.D = 0.0f;
        p.nx = 0.0f;
        p.ny = 0.0f;
        p.nz = 1.0f;
    }
    // 1/|t x n| for e1 (prop_e1)
    p.einv = fabsf(p.nz) < 0.9f ? rsqrtf(p.ny * p.ny + p.nx * p.nx) : rsqrtf(p.nz * p.nz + p.ny * p.ny);
    p.pxx = pi1.x;
    p.pxy = pi1.y;
    p.pxz = pi1.z;
    p.pyy = pi1.w;
    p.pyz = pi2.x;
    p.shear_c = 0.0f;
    if (cfg.include_shear) {
        if (cfg.neos_kind == 1) {
            // divided by p0 in the acceptance (try_once)
            p.shear_c = 1.0f / (2.0f * cf.z * T);
        } else if (cfg.neos_kind == 0) {
            p.shear_c = cf.x;
        } else {
            p.shear_c = 1.0f / (2.0f * T * T * (th2.x + th2.y));
        }
    }
    p.bi0 = p.b0 = p.b1 = p.b2 = 0.0f;
    if (cfg.include_bulk) {
        if (cfg.bulk_kind == 11) {
            const float Pi = th2.w;
            p.b0 = Pi * cf.x * m * m;
            p.b1 = Pi * cf.y * static_cast<float>(sp.baryon);
            p.b2 = Pi * cf.z;
        } else if (cfg.bulk_kind == 21 || cfg.bulk_kind == 1) {
            const float Pi = (cfg.bulk_kind == 1) ? th2.w / 0.197327053f : th2.w;
            p.bi0 = -cf.x * Pi * m * m / (3.0f * T);
            p.b1 = cf.x * Pi * cf.y / T;
        }
    }
    p.qx = p.qy = p.qz = p.pq = p.Bq = 0.0f;
    if (!kLean && cfg.include_diff) {
        const float ik = 1.0f / cf.w;
        p.qx = pi2.y * ik;
        p.qy = pi2.z * ik;
        p.qz = pi2.w * ik;
        p.pq = th2.z / (th2.x + th2.y);
        p.Bq = static_cast<float>(sp.baryon);
    }
    return true;
}

__device__ float compat_ratio(const Prop& p, float Et) {
    const float q = expf(-Et);
    float e = 1.0f, S1 = 0.0f, S2 = 0.0f;
#pragma unroll
    for (int n = 1; n <= 10; n++) {
        e *= q;
        S2 += e;
        S1 += ((p.sign == -1) || (n & 1)) ? e : -e;
    }
    const float finf = (p.sign == -1) ? q / (-expm1f(-Et)) : q / (1.0f + q);
    const float num = Et * Et * S2 + 2.0f * p.mut * Et * S1 + p.cpoly * finf;
    const float den = (Et * Et + 2.0f * p.mut * Et + p.cpoly) * finf;
    return num / den;
}

// The Bose proposal of bosons (the plain sampler's): |p| from
// (K^2 + 2 m~ K + m~^2/2) (e^-K + e^-a e^-2K + e^-2a e^-3K), i.e. p^2-weighted
// e^-E~ + e^-2E~ + e^-3E~, the first three terms of the Bose-Einstein series.
// Term n is a Gamma(3), Gamma(2), Gamma(1) mixture at rate n with weights
// e^-(n-1)a (2/n^3, 2 m~/n^2, m~^2/(2n)), i.e. e^-(n-1)a (2/n^3) (1, n m~,
// n^2 m~^2/4).  Against this proposal the statistics factor is
// f_BE / (e^-E~ + e^-2E~ + e^-3E~) = 1 / (1 - e^-3E~), largest at K = 0, so
// the try accepts with qa / (1 - e^-3E~), qa = 1 - e^-3a (for pions about 0.94
// on average, against 0.67 with the one-term proposal).  Fermions keep the
// one-term proposal (W1 = W12 = W).
__device__ __forceinline__ void prop_bose2(Prop& p) {
    p.W1 = p.W;
    p.W12 = p.W;
    p.r2 = 0.0f;
    if (p.sign != -1) return;
    const float ea = __expf(-p.a);
    p.W12 = p.W1 + 0.25f * ea * (1.0f + p.mt) * (1.0f + p.mt);
    p.W = p.W12 + (2.0f / 27.0f) * ea * ea * (1.0f + 1.5f * p.mt) * (1.0f + 1.5f * p.mt);
    p.r2 = 4.0f / ea;
    p.qa = p.a > 0.0167f ? 1.0f - ea * ea * ea : -expm1f(-3.0f * p.a);
}

// One proposal.  On acceptance fills the LRF momentum (p0, px, py, pz) and
// the uniform used for the rapidity of boost-invariant surfaces.  kBose2:
// the proposal of prop_bose2 (the plain sampler); otherwise the one-term
// proposal the learned sampler's densities assume.
template <int kMode = 0, bool kBose2 = false>
__device__ __forceinline__ bool try_once(const DevConfig& cfg, const Prop& p, const Unit& u,
                                         float4& pl, float& u_rap, unsigned& violations) {
    const uint32_t c3 = static_cast<uint32_t>(u.s) | (kTagTry << 16);
    const uint4 A = block(2u * u.t, u.i, u.eg, c3, cfg.key0, cfg.key1);
    const float sel = u01f(A.x) * p.W;
    float prod = u01f_pos(A.y);
    float K;
    if constexpr (kBose2) {
        // term n rescaled to weights (1, n m~, n^2 m~^2/4): Gamma(3) below 1,
        // Gamma(2) below 1 + n m~; the rescale is 1/2 for term 1, r2 = 4 e^a
        // for term 2 and 27 e^2a / 2 = (27/32) r2^2 for term 3
        const bool t2 = sel >= p.W1, t3 = sel >= p.W12;
        // (the small factor first: r2^2 alone can overflow for heavy bosons)
        const float s = t3 ? ((sel - p.W12) * p.r2) * (0.84375f * p.r2)
                           : (t2 ? (sel - p.W1) * p.r2 : 0.5f * sel);
        const float n = t3 ? 3.0f : (t2 ? 2.0f : 1.0f);
        if (s < 1.0f + n * p.mt) prod *= u01f_pos(A.z);
        if (s < 1.0f) prod *= u01f_pos(A.w);
        K = -logf(prod) * (t3 ? (1.0f / 3.0f) : (t2 ? 0.5f : 1.0f));
    } else {
        if (sel < p.w32) prod *= u01f_pos(A.z);
        if (sel < p.w3) prod *= u01f_pos(A.w);
        K = -logf(prod);
    }
    if (K > p.Kmax) return false;
    const uint4 B = block(2u * u.t + 1u, u.i, u.eg, c3, cfg.key0, cfg.key1);
    const float k2 = K * (K + 2.0f * p.mt);
    const float Et = K + p.mt;
    const float ptil = sqrtf(k2);
    const float a_pE = Et * ptil / (k2 + 0.5f * p.mt * p.mt);
    const float Etil = p.a + K;
    const float em = expf(-Etil);
    // 1 - e^-Etil (1 - e^-2Etil) from em where that is accurate (relative
    // error below 3e-6); expm1f near Bose condensation only
    float a_q;
    if (kBose2)
        a_q = (p.sign == -1) ? p.qa / (Etil > 0.0167f ? 1.0f - em * em * em : -expm1f(-3.0f * Etil))
                             : 1.0f / (1.0f + em);
    else
        a_q = (p.sign == -1) ? p.qa / (Etil > 0.05f ? 1.0f - em : -expm1f(-Etil))
                             : 1.0f / (1.0f + em);
    float a_c = 1.0f;
    if (kMode == 0 && p.compat) {
        a_c = compat_ratio(p, Etil) / p.rmax;
        if (a_c > 1.0f) {
            violations++;
            a_c = 1.0f;
        }
    }
    // direction: cos(alpha) from the density max(0, d0 + beta D cos(alpha))
    // (inverse CDF, stable root), azimuth uniform around n
    const float beta = ptil / Et;
    const float bD = beta * p.D;
    float c_lo = -1.0f, r_flux = 1.0f;
    if (bD > p.d0) {
        c_lo = -p.d0 / bD;
        const float s0 = p.d0 + p.D;
        r_flux = (p.d0 + bD) * (p.d0 + bD) / (beta * s0 * s0);
    } else if (p.D > p.d0) {
        const float s0 = p.d0 + p.D;
        r_flux = 4.0f * p.d0 * p.D / (s0 * s0);
    }
    const float a_lin = p.d0 + bD * c_lo;
    const float L = 1.0f - c_lo;
    const float uZ = u01f(B.x) * (a_lin * L + 0.5f * bD * L * L);
    const float cth = fminf(c_lo + 2.0f * uZ / (a_lin + sqrtf(a_lin * a_lin + 2.0f * bD * uZ)), 1.0f);
    const float sth = sqrtf(fmaxf(1.0f - cth * cth, 0.0f));
    float sphi, cphi;
    // azimuth in [-pi, pi), where the SFU's sine and cosine are accurate to 2^-20
    __sincosf(kTwoPiF * (u01f(B.y) - 0.5f), &sphi, &cphi);
    float e1x, e1y, e1z;
    prop_e1(p, e1x, e1y, e1z);
    const float e2x = p.ny * e1z - p.nz * e1y;
    const float e2y = p.nz * e1x - p.nx * e1z;
    const float e2z = p.nx * e1y - p.ny * e1x;
    const float T = p.T;
    const float pm = T * ptil;
    const float p0 = T * Et;
    const float px = pm * (cth * p.nx + sth * (cphi * e1x + sphi * e2x));
    const float py = pm * (cth * p.ny + sth * (cphi * e1y + sphi * e2y));
    const float pz = pm * (cth * p.nz + sth * (cphi * e1z + sphi * e2z));
    const float sgn = static_cast<float>(p.sign);
    const float f0 = em / (1.0f + sgn * em);
    const float one_m = 1.0f - sgn * f0;
    float df = 0.0f;
    if (cfg.include_shear) {
        const float Wf = px * px * p.pxx + 2.0f * px * py * p.pxy + 2.0f * px * pz * p.pxz +
                         py * py * p.pyy + 2.0f * py * pz * p.pyz + pz * pz * (-p.pxx - p.pyy);
        float ds = one_m * Wf * p.shear_c;
        if (cfg.neos_kind == 1) ds /= p0;
        df += ds;
    }
    if (cfg.include_bulk) {
        df += one_m * (p.bi0 / p0 + p.b0 + p.b1 * p0 + p.b2 * p0 * p0);
    }
    if (kMode != 1 && cfg.include_diff) {
        const float qf = -(px * p.qx + py * p.qy + pz * p.qz);
        df += one_m * (p.pq - p.Bq / p0) * qf;
    }
    const float fact2 = clamp01((1.0f + df) * 0.5f);
    const float acc = a_pE * a_q * a_c * r_flux * fact2;
    if (!(u01f(B.z) < acc)) return false;
    pl = make_float4(p0, px, py, pz);
    u_rap = u01f(B.w);
    return true;
}

// ---------------------------------------------------------------------------
// MC_sampling = 2: the reference's EmissionFunctionArray sampler
// (sample_using_dN_dxtdy_4all_particles_conventional and
// sample_momemtum_from_a_fluid_cell, src/emissionfunction.cpp:3273-3623,
// 4188-4309).  Per hadron a cell is drawn from the same per-species CDF as in
// FSSW; then pT is proposed from pT dpT on [0, pT_max], phi uniformly and
// y - eta_s uniformly in [-range, range] in the lab (Milne) frame, and the
// proposal is accepted with f0 p.dsigma tau (1 + delta f) / maximum, where the
// maximum is the reference's analytic upper bound of the emission function
// (estimate_maximum, src/emissionfunction.cpp:4309-4421).  After 5,000 tries
// the cell is drawn again (src/emissionfunction.cpp:3475-3480).

constexpr float kEfaInvE = 0.3678794f;   // the reference's cut for 1/e

// principal branch W0(x) for x >= -1/e: series about the branch point or a
// logarithmic start, then Halley iterations
__device__ float lambert_w0(float x) {
    if (x <= -0.36787944f) return -1.0f;
    float w;
    if (x < -0.25f) {
        const float pp = sqrtf(2.0f * (2.7182818f * x + 1.0f));
        w = -1.0f + pp * (1.0f + pp * (-1.0f / 3.0f + pp * (11.0f / 72.0f)));
    } else if (x < 3.0f) {
        w = log1pf(x) * (1.0f - 0.25f * log1pf(x) / (1.0f + log1pf(x)));
    } else {
        const float l1 = logf(x), l2 = logf(l1);
        w = l1 - l2 + l2 / l1;
    }
#pragma unroll
    for (int it = 0; it < 5; it++) {
        const float ew = expf(w);
        const float f = w * ew - x;
        const float wp1 = w + 1.0f;
        if (fabsf(wp1) < 1e-6f) break;
        w -= f / (ew * wp1 - (w + 2.0f) * f / (2.0f * wp1));
    }
    return w;
}

// max over E >= m of E^A f0(E) (estimate_ideal_maximum / the A = 2, 3 forms of
// estimate_shear_viscous_maximum and estimate_diffusion_maximum): the
// stationary point solves (beta E - A) exp(beta E - A) = sign A exp(beta mu - A)
__device__ float ea_f0_max(int sign, int A, float m, float T, float mu, float f0m) {
    const float iT = 1.0f / T;
    const float mA = m * m * (A == 3 ? m : (A == 2 ? 1.0f : 1.0f / m));   // m^A
    if (sign == 1) {
        float Emax = T * (lambert_w0(A * expf(iT * mu - A)) + A);
        if (Emax < m) Emax = m;
        const float eA = A == 1 ? Emax : (A == 2 ? Emax * Emax : Emax * Emax * Emax);
        return eA / (expf((Emax - mu) * iT) + sign);
    }
    const float rhs = A * expf(iT * mu - A);
    if (rhs > kEfaInvE) return mA * f0m;
    // z exp(-z) = rhs with z <= 1, i.e. z = -W0(-rhs)
    const float Emax = T * (A + lambert_w0(-rhs));
    if (Emax < m) return mA * f0m;
    const float eA = A == 1 ? Emax : (A == 2 ? Emax * Emax : Emax * Emax * Emax);
    return fmaxf(eA / (expf((Emax - mu) * iT) + sign), mA * f0m);
}

struct PropEfa {
    float tau, T, mu, m, bmax;     // bmax: the reference's maximum / (degen prefactor)
    float da0, da1, da2, da3, u0, u1, u2, u3;
    float pi00, pi01, pi02, pi03, pi11, pi12, pi13, pi22, pi23, pi33;
    float q0, q1, q2, q3;
    float shear_pref, bulk_c0, bulk_c1, bulkPi, qpref, ikappa;
    int sign, baryon;
};

// one (cell, species): the Milne cell and the maximum (estimate_maximum)
__device__ bool setup_efa(const DevConfig& cfg, const CellArrays& cells, const SpeciesDev& sp, int l,
                          PropEfa& p, bool keep_max) {
    const float4* rec = cells.rec + 8 * static_cast<int64_t>(l);
    const float4* mr = cells.milne + 6 * static_cast<int64_t>(l);
    const float4 pos = __ldg(rec), th = __ldg(rec + 3), th2 = __ldg(rec + 4), cf = __ldg(rec + 7);
    const float4 m0 = __ldg(mr), m1 = __ldg(mr + 1), m2 = __ldg(mr + 2), m3 = __ldg(mr + 3);
    const float4 m4 = __ldg(mr + 4), m5 = __ldg(mr + 5);
    p.tau = pos.x;
    p.T = th.x;
    p.m = sp.m_hi + sp.m_lo;
    p.mu = static_cast<float>(sp.baryon) * th.y + static_cast<float>(sp.strange) * th.z +
           static_cast<float>(sp.charge) * th.w;
    p.sign = sp.sign;
    p.baryon = sp.baryon;
    p.da0 = m0.x; p.da1 = m0.y; p.da2 = m0.z; p.da3 = m0.w;
    p.u0 = m1.x; p.u1 = m1.y; p.u2 = m1.z; p.u3 = m1.w;
    p.pi00 = m2.x; p.pi01 = m2.y; p.pi02 = m2.z; p.pi03 = m2.w;
    p.pi11 = m3.x; p.pi12 = m3.y; p.pi13 = m3.z; p.pi22 = m3.w;
    p.pi23 = m4.x; p.pi33 = m4.y; p.q0 = m4.z; p.q1 = m4.w;
    p.q2 = m5.x; p.q3 = m5.y;
    const float ep = th2.x + th2.y;
    p.shear_pref = cfg.include_shear ? 1.0f / (2.0f * p.T * p.T * ep) : 0.0f;
    p.bulkPi = cfg.include_bulk ? m5.z / 0.197327053f : 0.0f;   // fm^-4 (bulk_deltaf_kind 1)
    p.bulk_c0 = cf.x;
    p.bulk_c1 = cf.y;
    p.qpref = cfg.include_diff ? th2.z / ep : 0.0f;
    p.ikappa = cfg.include_diff ? 1.0f / cf.w : 0.0f;
    if (keep_max) return true;
    // estimate_maximum (src/emissionfunction.cpp:4309-4421)
    const float udsig = p.tau * (p.u0 * p.da0 + p.u1 * p.da1 + p.u2 * p.da2 + p.u3 * p.da3 / p.tau);
    const float dsig2 = p.tau * p.tau * (p.da0 * p.da0 - p.da1 * p.da1 - p.da2 * p.da2 -
                                         p.da3 * p.da3 / (p.tau * p.tau));
    const float dsigT = sqrtf(fabsf(dsig2 - udsig * udsig));
    const float dsig_all = fabsf(udsig) + dsigT;
    const float f0m = 1.0f / (expf((p.m - p.mu) / p.T) + p.sign);
    const float g_ideal = ea_f0_max(p.sign, 1, p.m, p.T, p.mu, f0m);
    float g = g_ideal;
    const float tmpf = p.sign == -1 ? 2.0f : 1.0f;
    if (cfg.include_shear) {
        const float tr = p.pi00 * p.pi00 + p.pi11 * p.pi11 + p.pi22 * p.pi22 + p.pi33 * p.pi33 -
                         2.f * p.pi01 * p.pi01 - 2.f * p.pi02 * p.pi02 - 2.f * p.pi03 * p.pi03 +
                         2.f * p.pi12 * p.pi12 + 2.f * p.pi13 * p.pi13 + 2.f * p.pi23 * p.pi23;
        const float pi_size = sqrtf(fmaxf(tr, 0.0f)) / ep;
        g += ea_f0_max(p.sign, 3, p.m, p.T, p.mu, f0m) * tmpf / (2.0f * p.T * p.T) * pi_size;
    }
    if (cfg.include_bulk)
        g += fabsf(p.bulkPi * p.bulk_c0) * p.m * p.m / p.T / 3.0f * f0m * (1.0f - p.sign * f0m);
    if (cfg.include_diff) {
        const float qsq = p.q0 * p.q0 - p.q1 * p.q1 - p.q2 * p.q2 - p.q3 * p.q3;
        float gq = p.qpref * ea_f0_max(p.sign, 2, p.m, p.T, p.mu, f0m);
        if (p.baryon > 0) gq += p.baryon * g_ideal;
        g += gq * tmpf * sqrtf(fabsf(qsq)) * p.ikappa;
    }
    p.bmax = dsig_all * g;
    return true;
}

// one lab-frame proposal (sample_momemtum_from_a_fluid_cell): pl = (pT, phi,
// y - eta_s, -) on acceptance, u_rap the uniform of the rapidity draw
__device__ __forceinline__ bool try_efa(const DevConfig& cfg, const PropEfa& p, const Unit& u,
                                        float4& pl, float& u_rap, unsigned& violations) {
    const uint32_t c3 = static_cast<uint32_t>(u.s) | (kTagEfa << 16);
    const uint4 A = block(u.t, u.i, u.eg, c3, cfg.key0, cfg.key1);
    const float pT = sqrtf(cfg.pt_max * cfg.pt_max * u01f(A.x));
    const float phi = 2.0f * 3.14159265f * u01f(A.y);
    const float yme = (1.0f - 2.0f * u01f(A.z)) * cfg.yme_range;
    const float mT = sqrtf(p.m * p.m + pT * pT);
    float sphi, cphi;
    sincosf(phi, &sphi, &cphi);
    const float px = pT * cphi, py = pT * sphi;
    const float p0 = mT * coshf(yme), p3 = mT * sinhf(yme);
    const float pdotu = p0 * p.u0 - px * p.u1 - py * p.u2 - p3 * p.u3;
    const float f0 = 1.0f / (expf((pdotu - p.mu) / p.T) + p.sign);
    const float pdsig = p0 * p.da0 + px * p.da1 + py * p.da2 + p3 * p.da3 / p.tau;
    const float one_m = 1.0f - p.sign * f0;
    float df = 0.0f;
    if (cfg.include_shear) {
        const float W = p0 * p0 * p.pi00 - 2.f * p0 * px * p.pi01 - 2.f * p0 * py * p.pi02 -
                        2.f * p0 * p3 * p.pi03 + px * px * p.pi11 + 2.f * px * py * p.pi12 +
                        2.f * px * p3 * p.pi13 + py * py * p.pi22 + 2.f * py * p3 * p.pi23 +
                        p3 * p3 * p.pi33;
        df += one_m * W * p.shear_pref;
    }
    if (cfg.include_bulk) {
        const float EoT = pdotu / p.T, moT = p.m / p.T;
        df += -one_m * p.bulk_c0 * (moT * moT / (3.0f * EoT) - p.bulk_c1 * EoT) * p.bulkPi;
    }
    if (cfg.include_diff) {
        const float qf = p0 * p.q0 - px * p.q1 - py * p.q2 - p3 * p.q3;
        df += one_m * (p.qpref - p.baryon / pdotu) * qf * p.ikappa;
    }
    float resize = 1.0f;
    if (cfg.restrict_df) resize = fminf(1.0f, cfg.df_max_ratio / (fabsf(df) + 1e-10f));
    const float result = f0 * pdsig * p.tau * (1.0f + df * resize);
    const float acc = result / p.bmax;
    if (acc > 1.0f) violations++;
    if (!(u01f(A.w) < acc)) return false;
    pl = make_float4(pT, phi, yme, 0.0f);
    u_rap = 0.0f;
    if (cfg.hydro_mode != 2) {
        const uint4 B = block(u.t, u.i, u.eg, static_cast<uint32_t>(u.s) | (kTagEfaRap << 16),
                              cfg.key0, cfg.key1);
        u_rap = u01f(B.x);
    }
    return true;
}

// ---------------------------------------------------------------------------
// Learned proposal.  The target density of a (cell, species) pair in the
// rest frame, per dK dOmega with K = (E - m)/T, is P(K, n) a(K, n): P is the
// plain proposal above (Gamma mixture in K, flux-linear direction) and a its
// acceptance (quantum statistics, pE/(E^2 - m^2/2), flux remainder, delta f),
// so both samplers accept exactly the reference's p^2 f(E) x weight.  The
// learned sampler proposes from q = alpha Q + (1 - alpha) P, Q the network's
// mixture, and accepts with P a / (M q); M is the pair's envelope constant
// (pair_prepare_kernel).  A ratio above 1 means M was too small there; such
// proposals are counted (learned_violations).

constexpr float kTwoPi = 6.283185307179586f;

// plain proposal density P and acceptance a at (K, n); false where the
// target is zero (K beyond the momentum table, p.dsigma < 0).  pl receives
// the rest-frame four-momentum.
__device__ __forceinline__ bool plain_target(const DevConfig& cfg, const Prop& p, float K, float nx,
                                             float ny, float nz, float& P, float& a, float4& pl) {
    if (!(K > 0.0f) || K > p.Kmax) return false;
    const float k2 = K * (K + 2.0f * p.mt);
    const float Et = K + p.mt;
    const float ptil = sqrtf(k2);
    const float beta = ptil / Et;
    const float bD = beta * p.D;
    float c_lo = -1.0f, r_flux = 1.0f;
    if (bD > p.d0) {
        c_lo = -p.d0 / bD;
        const float s0 = p.d0 + p.D;
        r_flux = (p.d0 + bD) * (p.d0 + bD) / (beta * s0 * s0);
    } else if (p.D > p.d0) {
        const float s0 = p.d0 + p.D;
        r_flux = 4.0f * p.d0 * p.D / (s0 * s0);
    }
    const float cosa = nx * p.nx + ny * p.ny + nz * p.nz;
    if (cosa < c_lo) return false;
    const float a_lin = p.d0 + bD * c_lo;
    const float L = 1.0f - c_lo;
    const float Zd = a_lin * L + 0.5f * bD * L * L;
    const float PK = (K * K + 2.0f * p.mt * K + 0.5f * p.mt * p.mt) * expf(-K) / p.W;
    P = PK * fmaxf(p.d0 + bD * cosa, 0.0f) / (kTwoPi * Zd);
    const float a_pE = Et * ptil / (k2 + 0.5f * p.mt * p.mt);
    const float Etil = p.a + K;
    const float em = expf(-Etil);
    const float a_q = (p.sign == -1) ? p.qa / (-expm1f(-Etil)) : 1.0f / (1.0f + em);
    const float a_c = p.compat ? fminf(compat_ratio(p, Etil) / p.rmax, 1.0f) : 1.0f;
    const float T = p.T;
    const float pm = T * ptil;
    const float p0 = T * Et;
    const float px = pm * nx, py = pm * ny, pz = pm * nz;
    const float sgn = static_cast<float>(p.sign);
    const float f0 = em / (1.0f + sgn * em);
    const float one_m = 1.0f - sgn * f0;
    float df = 0.0f;
    if (cfg.include_shear) {
        const float Wf = px * px * p.pxx + 2.0f * px * py * p.pxy + 2.0f * px * pz * p.pxz +
                         py * py * p.pyy + 2.0f * py * pz * p.pyz + pz * pz * (-p.pxx - p.pyy);
        float ds = one_m * Wf * p.shear_c;
        if (cfg.neos_kind == 1) ds /= p0;
        df += ds;
    }
    if (cfg.include_bulk) df += one_m * (p.bi0 / p0 + p.b0 + p.b1 * p0 + p.b2 * p0 * p0);
    if (cfg.include_diff) {
        const float qf = -(px * p.qx + py * p.qy + pz * p.qz);
        df += one_m * (p.pq - p.Bq / p0) * qf;
    }
    a = a_pE * a_q * a_c * r_flux * clamp01((1.0f + df) * 0.5f);
    pl = make_float4(p0, px, py, pz);
    return true;
}

// a pair record's float4 j: through the read-only cache (global records) or
// a plain load (records staged in shared memory)
template <bool kShared>
__device__ __forceinline__ float4 rec4(const float* lp, int j) {
    if (kShared) return reinterpret_cast<const float4*>(lp)[j];
    return __ldg(reinterpret_cast<const float4*>(lp) + j);
}
template <bool kShared>
__device__ __forceinline__ float rec1(const float* lp, int j) {
    if (kShared) return lp[j];
    return __ldg(lp + j);
}

// the network's mixture density Q(K, n) per dK dOmega from a pair record
template <bool kShared = false>
__device__ __forceinline__ float learned_density(const float* __restrict__ lp, float K, float nx,
                                                 float ny, float nz) {
    const float lK = logf(K);
    float q = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float4 c = rec4<kShared>(lp, 2 * k);
        const float4 v = rec4<kShared>(lp, 2 * k + 1);
        const float d = (lK - c.z) / c.w;
        q += expf(c.y - 0.5f * d * d + v.x * nx + v.y * ny + v.z * nz);
    }
    return q / K;
}

// unit vector n around the pair's axis: frame (e1, e2) perpendicular to m
__device__ __forceinline__ void around(float mx, float my, float mz, float c, float sphi,
                                       float cphi, float& nx, float& ny, float& nz) {
    float tx = 0.f, tz = 0.f;
    if (fabsf(mz) < 0.9f) tz = 1.f; else tx = 1.f;
    float ex = -tz * my, ey = tz * mx - tx * mz, ez = tx * my;
    const float inv = rsqrtf(ex * ex + ey * ey + ez * ez);
    ex *= inv;
    ey *= inv;
    ez *= inv;
    const float fx = my * ez - mz * ey, fy = mz * ex - mx * ez, fz = mx * ey - my * ex;
    const float s = sqrtf(fmaxf(1.0f - c * c, 0.0f));
    nx = c * mx + s * (cphi * ex + sphi * fx);
    ny = c * my + s * (cphi * ey + sphi * fy);
    nz = c * mz + s * (cphi * ez + sphi * fz);
}

// one proposal from the network's mixture Q (from_q) or from the plain
// proposal P, from the uniforms A.y .. B.z (A.x and B.w are the caller's);
// false when it falls outside the support
template <bool kShared = false>
__device__ __forceinline__ bool propose_mixture(const Prop& p, const float* __restrict__ lp,
                                                bool from_q, const uint4& A, const uint4& B,
                                                float& K, float& nx, float& ny, float& nz) {
    if (from_q) {
        const float uc = u01f(A.y);
        int k = 0;
        while (k < 7 && uc >= rec1<kShared>(lp, 8 * k)) k++;
        const float4 c = rec4<kShared>(lp, 2 * k);
        const float4 v = rec4<kShared>(lp, 2 * k + 1);
        const float uz = (static_cast<float>(A.z >> 8) + 0.5f) * (1.0f / 16777216.0f);
        const float z = 1.4142135623730951f * erfinvf(2.0f * uz - 1.0f);
        K = expf(c.z + c.w * z);
        const float kap = v.w;
        float mx = 0.f, my = 0.f, mz = 1.f;
        if (kap > 1e-6f) {
            mx = v.x / kap;
            my = v.y / kap;
            mz = v.z / kap;
        }
        const float uw = u01f(A.w);
        const float w = kap < 1e-4f ? 2.0f * uw - 1.0f
                                    : fmaxf(-1.0f, 1.0f + log1pf((1.0f - uw) * expm1f(-2.0f * kap)) / kap);
        float sphi, cphi;
        __sincosf(kTwoPiF * (u01f(B.y) - 0.5f), &sphi, &cphi);
        around(mx, my, mz, fminf(w, 1.0f), sphi, cphi, nx, ny, nz);
        return true;
    }
    const float sel = u01f(A.y) * p.W;
    float prod = u01f_pos(A.z);
    if (sel < p.w32) prod *= u01f_pos(A.w);
    if (sel < p.w3) prod *= u01f_pos(B.x);
    K = -logf(prod);
    if (K > p.Kmax) return false;
    const float k2 = K * (K + 2.0f * p.mt);
    const float beta = sqrtf(k2) / (K + p.mt);
    const float bD = beta * p.D;
    const float c_lo = bD > p.d0 ? -p.d0 / bD : -1.0f;
    const float a_lin = p.d0 + bD * c_lo;
    const float L = 1.0f - c_lo;
    const float uZ = u01f(B.y) * (a_lin * L + 0.5f * bD * L * L);
    const float cth = fminf(c_lo + 2.0f * uZ / (a_lin + sqrtf(a_lin * a_lin + 2.0f * bD * uZ)), 1.0f);
    float sphi, cphi;
    __sincosf(kTwoPiF * (u01f(B.z) - 0.5f), &sphi, &cphi);
    around(p.nx, p.ny, p.nz, cth, sphi, cphi, nx, ny, nz);
    return true;
}

// excess-branch bound c >= sup (a - M q / P) = 1 - M (1 - alpha), since
// a <= 1 and q / P >= 1 - alpha; the margin covers the FP32 rounding of a
constexpr float kExcessMargin = 1e-4f;
__device__ __forceinline__ float excess_bound(float M, float alpha) {
    return fmaxf(0.0f, 1.0f + kExcessMargin - M * (1.0f - alpha));
}

// One learned proposal and its accept step, for the target t = P a of the
// plain sampler and the envelope E = M q, q = alpha Q + (1 - alpha) P.
// Exact mode (cfg.lexact): with probability M / (M + c) the mixture branch
// (x from q, accepted with min(1, t / E)), else the excess branch (x from P,
// accepted with (t - E) / (c P), c = excess_bound).  Accepted density per
// try: [min(t, E) + (t - E)+] / (M + c) = t / (M + c), for any M: exact
// rejection whatever the envelope's quality.  A ratio above 1 in the
// mixture branch is then not an error: the excess branch supplies the mass
// min() drops there (counted in over_one); an excess-branch ratio above 1
// would mean c < sup (a - M q / P), and is counted as a violation.
// Without lexact: the mixture branch alone, ratios above 1 counted.
struct LearnedTryStats {
    unsigned viol = 0, excess_tries = 0, excess_hadrons = 0, over_one = 0;
};
__device__ __forceinline__ bool try_learned(const DevConfig& cfg, const Prop& p, const Unit& u,
                                            const float* __restrict__ lp, float4& pl, float& u_rap,
                                            LearnedTryStats& ls) {
    const uint32_t c3 = static_cast<uint32_t>(u.s) | (kTagLearn << 16);
    const uint4 A = block(2u * u.t, u.i, u.eg, c3, cfg.key0, cfg.key1);
    const uint4 B = block(2u * u.t + 1u, u.i, u.eg, c3, cfg.key0, cfg.key1);
    const float M = __ldg(lp + 56);
    const float alpha = cfg.lalpha;
    const float c = cfg.lexact ? excess_bound(M, alpha) : 0.0f;
    // one uniform picks the branch and, within the mixture branch, Q or P
    const float sel = u01f(A.x) * (M + c);
    const bool excess = sel < c;
    const bool from_q = !excess && (sel - c) < alpha * M;
    ls.excess_tries += excess;
    float K, nx, ny, nz, P, a;
    if (!propose_mixture(p, lp, from_q, A, B, K, nx, ny, nz)) return false;
    if (!plain_target(cfg, p, K, nx, ny, nz, P, a, pl)) return false;
    const float Q = learned_density(lp, K, nx, ny, nz);
    const float E = M * (alpha * Q + (1.0f - alpha) * P);
    float r;
    if (excess) {
        r = (P * a - E) / (c * P);
        if (r > 1.0f) ls.viol++;
    } else {
        r = P * a / E;
        if (r > 1.0f) {
            if (cfg.lexact) ls.over_one++; else ls.viol++;
        }
    }
    if (!(u01f(B.w) < r)) return false;
    ls.excess_hadrons += excess;
    u_rap = 0.0f;
    if (cfg.hydro_mode != 2) {
        const uint4 C = block(u.t, u.i, u.eg, static_cast<uint32_t>(u.s) | (kTagLearnRap << 16),
                              cfg.key0, cfg.key1);
        u_rap = u01f(C.x);
    }
    return true;
}

__device__ __forceinline__ void write_hadron(HadronRec* out, int64_t slot, int pid, float mass,
                                             float E, float px, float py, float pz, float t,
                                             float x, float y, float z) {
    // 40-byte records are 8-byte aligned: five 8-byte stores
    float2* o = reinterpret_cast<float2*>(out + slot);
    o[0] = make_float2(__int_as_float(pid), mass);
    o[1] = make_float2(E, px);
    o[2] = make_float2(py, pz);
    o[3] = make_float2(t, x);
    o[4] = make_float2(y, z);
}

// kMode 1, 2 (lean): u and the position come from the lean sampler's record,
// whose position of a 3+1D cell is already (t, x, y, z)
template <int kMode = 0>
__device__ void emit(const DevConfig& cfg, const CellArrays& cells, const Prop& p, int l, int pid,
                     float4 pl, float u_rap, HadronRec* out, int64_t slot) {
    constexpr bool kLean = kMode != 0;
    const float4* rec = (kLean ? cells.srec : cells.rec) + 8 * static_cast<int64_t>(l);
    const float4 u = __ldg(rec + (kLean ? 1 : 2));
    const float4 pos = __ldg(rec);
    const float pdu = pl.y * u.y + pl.z * u.z + pl.w * u.w;
    const float c = pdu / (u.x + 1.0f) + pl.x;
    const float lx = pl.y + c * u.y;
    const float ly = pl.z + c * u.z;
    const float lz = pl.w + c * u.w;
    const float mT2 = p.m * p.m + lx * lx + ly * ly;
    float eta_s, pz, E;
    if (cfg.hydro_mode == 2) {
        eta_s = pos.w;
        pz = lz;
        E = sqrtf(mT2 + lz * lz);
        if (kLean) {
            write_hadron(out, slot, pid, p.m, E, lx, ly, pz, pos.x, pos.y, pos.z, pos.w);
            return;
        }
    } else {
        const float mT = sqrtf(mT2);
        const float rap = cfg.y_lb + (cfg.y_rb - cfg.y_lb) * u_rap;
        const float y = asinhf(lz / mT);
        eta_s = rap - (y - pos.w);
        float sr, cr;
        sr = sinhf(rap);
        cr = coshf(rap);
        pz = mT * sr;
        E = mT * cr;
    }
    write_hadron(out, slot, pid, p.m, E, lx, ly, pz, pos.x * coshf(eta_s), pos.y, pos.z,
                 pos.x * sinhf(eta_s));
}

// add_one_sampled_particle of the EmissionFunctionArray path
// (src/emissionfunction.cpp:4423-4475): rapidity y = (y - eta_s) + eta_s,
// eta_s the cell's (3+1D) or drawn from a uniform rapidity (boost invariant)
__device__ void emit_efa(const DevConfig& cfg, const CellArrays& cells, const PropEfa& p, int l,
                         int pid, float4 pl, float u_rap, HadronRec* out, int64_t slot) {
    const float4 pos = __ldg(cells.rec + 8 * static_cast<int64_t>(l));
    const float pT = pl.x, yme = pl.z;
    float eta_s = pos.w;
    if (cfg.hydro_mode != 2) eta_s = cfg.y_lb + (cfg.y_rb - cfg.y_lb) * u_rap - yme;
    const float y = yme + eta_s;
    float sphi, cphi;
    sincosf(pl.y, &sphi, &cphi);
    const float mT = sqrtf(p.m * p.m + pT * pT);
    write_hadron(out, slot, pid, p.m, mT * coshf(y), pT * cphi, pT * sphi, mT * sinhf(y),
                 pos.x * coshf(eta_s), pos.y, pos.z, pos.x * sinhf(eta_s));
}

// the two samplers behind one work loop: FSSW (Prop) and the lab-frame
// EmissionFunctionArray sampler (PropEfa)
template <int kAlg> struct PropOf { using type = Prop; };
template <> struct PropOf<2> { using type = PropEfa; };

// bose2: the hadron takes the plain proposal (prop_bose2); false for those
// of the learned proposal, whose densities assume the one-term proposal
template <int kMode>
__device__ __forceinline__ bool setup_any(const DevConfig& cfg, const CellArrays& cells,
                                          const SpeciesDev& sp, int l, Prop& p, bool, bool bose2) {
    const bool ok = setup_prop<kMode>(cfg, cells, sp, l, p);
    if (bose2) prop_bose2(p);
    return ok;
}
template <int kMode>
__device__ __forceinline__ bool setup_any(const DevConfig& cfg, const CellArrays& cells,
                                          const SpeciesDev& sp, int l, PropEfa& p, bool keep_max, bool) {
    return setup_efa(cfg, cells, sp, l, p, keep_max);
}
template <int kMode, bool kBose2>
__device__ __forceinline__ bool try_any(const DevConfig& cfg, const Prop& p, const Unit& u, float4& pl,
                                        float& u_rap, unsigned& viol) {
    return try_once<kMode, kBose2>(cfg, p, u, pl, u_rap, viol);
}
template <int kMode, bool kBose2>
__device__ __forceinline__ bool try_any(const DevConfig& cfg, const PropEfa& p, const Unit& u,
                                        float4& pl, float& u_rap, unsigned& viol) {
    return try_efa(cfg, p, u, pl, u_rap, viol);
}
template <int kMode>
__device__ __forceinline__ void emit_any(const DevConfig& cfg, const CellArrays& cells, const Prop& p,
                                         int l, int pid, float4 pl, float u_rap, HadronRec* out,
                                         int64_t slot) {
    emit<kMode>(cfg, cells, p, l, pid, pl, u_rap, out, slot);
}
template <int kMode>
__device__ __forceinline__ void emit_any(const DevConfig& cfg, const CellArrays& cells,
                                         const PropEfa& p, int l, int pid, float4 pl, float u_rap,
                                         HadronRec* out, int64_t slot) {
    emit_efa(cfg, cells, p, l, pid, pl, u_rap, out, slot);
}

// Cell of every hadron's first draw (redraw 0), one warp per work item in
// species-major order.  Each lane runs independent searches, so the latency
// of the guide and CDF reads overlaps across many warps; the sampler then
// starts each hadron from cell_of[slot] instead of a dependent search.
constexpr int kAssignThreads = 256;

__global__ void __launch_bounds__(kAssignThreads)
cell_assign_kernel(DevConfig cfg_in, const unsigned long long* __restrict__ cdf,
                   const int32_t* __restrict__ guide,
                   const unsigned long long* __restrict__ qtot, const int64_t* __restrict__ offsets,
                   const int64_t* __restrict__ item_off, const int32_t* __restrict__ item_seg,
                   int64_t k_begin, int64_t k_end, const SpeciesDev* __restrict__ species,
                   int32_t* __restrict__ cell_of, const int64_t* __restrict__ k_end_dev) {
    const DevConfig cfg = with_run_keys(cfg_in);
    if (k_end_dev) k_end = *k_end_dev;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t n_warps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t k = k_begin + warp; k < k_end; k += n_warps) {
        const int q = item_seg[k];
        const int64_t j = k - item_off[q];
        int e, s;
        item_decode(cfg, q, e, s);
        const int64_t seg = static_cast<int64_t>(e) * cfg.n_species + s;
        const int64_t base = offsets[seg];
        const int mult = records_per_draw(cfg, species[s]);
        const int64_t draws = (offsets[seg + 1] - base) / mult;
        const int64_t d_begin = j * cfg.item_size;
        const int64_t d_end = min(d_begin + cfg.item_size, draws);
        const int b = cfg.ev_surf[e];
        const SurfSeg sg = cfg.surf[b];
        const unsigned long long* row = cdf + sg.cdf_base + static_cast<int64_t>(s) * (sg.n + 1);
        const int32_t* gd = guide + sg.guide_base + static_cast<int64_t>(s) * ((int64_t(1) << sg.g) + 1);
        const unsigned long long Q = qtot[b * cfg.n_species + s];
        const uint32_t eg = cfg.event_offset + static_cast<uint32_t>(e);
        const uint32_t c3 = static_cast<uint32_t>(s) | (kTagCell << 16);
        // 64 draws at a time: each lane takes the pair (2k, 2k + 1), whose
        // 64-bit uniforms are the two halves of one Philox block with counter
        // k (d_begin is even: item sizes are multiples of 32), and issues both
        // guide lookups before either search, so their latencies overlap
        for (int64_t d_sub = d_begin; d_sub < d_end; d_sub += kAssignSub) {
        const int64_t d0 = d_sub + 2 * lane, d1 = d0 + 1;
        const bool v0 = d0 < d_end, v1 = d1 < d_end;
        unsigned long long r0 = 0, r1 = 0;
        if (v0) {
            const uint4 w = block(0u, static_cast<uint32_t>(d0 >> 1), eg, c3, cfg.key0, cfg.key1);
            r0 = (static_cast<unsigned long long>(w.x) << 32) | static_cast<unsigned long long>(w.y);
            r1 = (static_cast<unsigned long long>(w.z) << 32) | static_cast<unsigned long long>(w.w);
        }
        const int last = static_cast<int>(sg.n - 1);
        const unsigned j0 = static_cast<unsigned>(r0 >> (64 - sg.g));
        const unsigned j1 = static_cast<unsigned>(r1 >> (64 - sg.g));
        int lo0 = 0, hi0 = 0, lo1 = 0, hi1 = 0;
        if (v0) {
            lo0 = __ldg(gd + j0);
            hi0 = __ldg(gd + j0 + 1);
        }
        if (v1) {
            lo1 = __ldg(gd + j1);
            hi1 = __ldg(gd + j1 + 1);
        }
        const unsigned long long q0 = __umul64hi(r0, Q), q1 = __umul64hi(r1, Q);
        lo0 = min(max(lo0, 0), last);
        hi0 = min(max(hi0, lo0), last);
        lo1 = min(max(lo1, 0), last);
        hi1 = min(max(hi1, lo1), last);
        // buckets of up to kAssignSpan cells: the candidates' CDF entries are
        // read at once and counted (C is nondecreasing and C[lo] <= v, so the
        // cell is lo + #{i in 1..w : C[lo + i] <= v}, what the binary search
        // below finds): one dependent read instead of a chain of them
        {
            const int w0 = hi0 - lo0, w1 = hi1 - lo1;
            unsigned long long a0[kAssignSpan], a1[kAssignSpan];
#pragma unroll
            for (int i = 0; i < kAssignSpan; i++) {
                a0[i] = (w0 <= kAssignSpan && i < w0) ? __ldg(row + lo0 + 1 + i) : ~0ull;
                a1[i] = (w1 <= kAssignSpan && i < w1) ? __ldg(row + lo1 + 1 + i) : ~0ull;
            }
            int k0 = 0, k1 = 0;
#pragma unroll
            for (int i = 0; i < kAssignSpan; i++) {
                k0 += a0[i] <= q0;
                k1 += a1[i] <= q1;
            }
            if (w0 <= kAssignSpan) {
                lo0 += k0;
                hi0 = lo0;
            }
            if (w1 <= kAssignSpan) {
                lo1 += k1;
                hi1 = lo1;
            }
        }
        while (lo0 < hi0 || lo1 < hi1) {
            const int m0 = (lo0 + hi0 + 1) >> 1, m1 = (lo1 + hi1 + 1) >> 1;
            const unsigned long long c0 = lo0 < hi0 ? __ldg(row + m0) : 0ull;
            const unsigned long long c1 = lo1 < hi1 ? __ldg(row + m1) : 0ull;
            if (lo0 < hi0) {
                if (c0 <= q0) lo0 = m0; else hi0 = m0 - 1;
            }
            if (lo1 < hi1) {
                if (c1 <= q1) lo1 = m1; else hi1 = m1 - 1;
            }
        }
        if (v0) cell_of[base - cfg.slot_base + d0 * mult] = static_cast<int32_t>(sg.c0) + lo0;
        if (v1) cell_of[base - cfg.slot_base + d1 * mult] = static_cast<int32_t>(sg.c0) + lo1;
        }
    }
}

constexpr int kSampleThreads = 256;

// kLcc: local_charge_conservation pairs (a separate instantiation, so the
// common case carries none of the pair state); kMode (setup_prop): 0 every
// configuration, 1 FSSW without diffusion and without the compat-fermion
// correction (both compile out, which frees registers), 2 the same with
// diffusion; 1 and 2 read the prologue's lean cell records (the learned
// proposal's plain component uses the same Prop fields)
template <bool kLcc, bool kLearned, int kAlg, int kMode>
__global__ void __launch_bounds__(kSampleThreads, 3)
sampler_kernel(DevConfig cfg_in, CellArrays cells, const SpeciesDev* __restrict__ species,
               const int32_t* __restrict__ pids, const unsigned long long* __restrict__ cdf,
               const int32_t* __restrict__ guide,
               const unsigned long long* __restrict__ qtot, const int64_t* __restrict__ offsets,
               const int64_t* __restrict__ item_off, const int32_t* __restrict__ item_seg,
               int64_t k_begin, int64_t k_end, int32_t* __restrict__ cell_of,
               HadronRec* __restrict__ out,
               unsigned long long* __restrict__ work_counter, SampleCounters* __restrict__ ctrs,
               const int64_t* __restrict__ k_end_dev) {
    const DevConfig cfg = with_run_keys(cfg_in);
    if (k_end_dev) k_end = *k_end_dev;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    // the three-term Bose proposal (prop_bose2) in the lean mode without
    // diffusion; the other modes keep the one-term proposal, whose fewer
    // registers spill less there (finite density: sample phase 30.3 ms with
    // the Bose terms, 28.3 ms without)
    constexpr bool kBose = kAlg == 4 && kMode == 1;
    // the warp's current work item: units [next, end) of species cur_s in event cur_e
    // draws [next, end), records from seg_base; a segment's draws are
    // counted by an int32, so draw indices fit in an int
    int next = 0, end = 0;
    int64_t seg_base = 0;
    int cur_s = 0, cur_e = 0, cur_mult = 1;
    bool exhausted = false;
    bool active = false;
    Unit u;
    typename PropOf<kAlg>::type p;
    // per-thread counts (a thread makes far fewer than 2^32 tries in a launch)
    unsigned n_tries = 0, n_redraws = 0, n_fail = 0;
    unsigned n_viol = 0;
    unsigned n_ltries = 0, n_lhad = 0;
    LearnedTryStats lts;

    for (;;) {
        // hand out units to the lanes that have none
        for (;;) {
            const unsigned need = __ballot_sync(FULL, !active);
            if (need == 0 || exhausted) break;
            if (next >= end) {
                long long k = 0;
                if (lane == 0) k = k_begin + static_cast<long long>(atomicAdd(work_counter, 1ull));
                k = __shfl_sync(FULL, k, 0);
                if (k >= k_end) {
                    exhausted = true;
                    break;
                }
                const int q = item_seg[k];
                const int64_t j = k - item_off[q];
                item_decode(cfg, q, cur_e, cur_s);
                const int64_t seg = static_cast<int64_t>(cur_e) * cfg.n_species + cur_s;
                seg_base = offsets[seg];
                cur_mult = kLcc ? records_per_draw(cfg, species[cur_s]) : 1;
                const int64_t first = j * cfg.item_size;
                next = static_cast<int>(first);
                end = static_cast<int>(min(first + cfg.item_size, (offsets[seg + 1] - seg_base) / cur_mult));
            }
            const int avail = end - next;
            const int rank = __popc(need & ((1u << lane) - 1u));
            if (!active && rank < avail) {
                const int64_t d = next + rank;
                u.s = cur_s;
                u.slot = seg_base - cfg.slot_base + d * cur_mult;
                u.i = static_cast<uint32_t>(d);
                u.mult = cur_mult;
                u.phase = 0;
                u.eg = cfg.event_offset + static_cast<uint32_t>(cur_e);
                u.redraw = 0;
                u.t = 0;
                u.tries_cell = 0;
                u.cell = -1;
                u.lp = nullptr;
                active = true;
            }
            next += min(__popc(need), avail);
        }
        if (__ballot_sync(FULL, active) == 0) break;
        if (active) {
            if (kLcc && u.phase == 1 && u.tries_cell >= cfg.max_tries) {
                // the partner stays in its pair's cell (the reference retries there)
                u.redraw++;
                n_redraws++;
                u.tries_cell = 0;
                if (u.redraw > cfg.max_redraws) {
                    write_hadron(out, u.slot + 1, 0, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f);
                    n_fail++;
                    active = false;
                    continue;
                }
            } else if (u.cell < 0 || u.tries_cell >= cfg.max_tries) {
                if (u.cell >= 0) {
                    u.redraw++;
                    n_redraws++;
                }
                if (u.redraw > cfg.max_redraws) {
                    for (int q = 0; q < (kLcc ? u.mult : 1); q++)
                        write_hadron(out, u.slot + q, 0, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f);
                    n_fail += kLcc ? u.mult : 1;
                    active = false;
                    continue;
                }
                int l;
                if (u.redraw == 0) {
                    l = cell_of[u.slot];
                } else {
                    const uint4 w = block(static_cast<uint32_t>(u.redraw), u.i, u.eg,
                                          static_cast<uint32_t>(u.s) | (kTagCell << 16), cfg.key0,
                                          cfg.key1);
                    const unsigned long long r = (static_cast<unsigned long long>(w.x) << 32) |
                                                 static_cast<unsigned long long>(w.y);
                    const int b = cfg.ev_surf[u.eg - cfg.event_offset];
                    const SurfSeg sg = cfg.surf[b];
                    l = static_cast<int>(sg.c0) +
                        cell_search(cdf + sg.cdf_base + static_cast<int64_t>(u.s) * (sg.n + 1), sg.n,
                                    guide + sg.guide_base +
                                        static_cast<int64_t>(u.s) * ((int64_t(1) << sg.g) + 1),
                                    sg.g, qtot[b * cfg.n_species + u.s], r);
                }
                u.cell = l;
                u.tries_cell = 0;
                if (kLearned) {
                    const int sl = cfg.lslot[u.s];
                    u.lp = sl >= 0 ? cfg.lpairs + (static_cast<int64_t>(sl) * cfg.n_cells + l) * kPairFloats
                                   : nullptr;
                }
                if (!setup_any<kMode>(cfg, cells, species[u.s], l, p, false, kBose && (!kLearned || !u.lp))) {
                    atomicCAS(&ctrs->error_code, 0, 1);
                    ctrs->error_species = u.s;
                    for (int q = 0; q < (kLcc ? u.mult : 1); q++)
                        write_hadron(out, u.slot + q, 0, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f);
                    n_fail += kLcc ? u.mult : 1;
                    active = false;
                    continue;
                }
            }
            float4 pl;
            float u_rap;
            bool ok;
            if constexpr (kLearned) {
                if (u.lp) {
                    ok = try_learned(cfg, p, u, u.lp, pl, u_rap, lts);
                    n_ltries++;
                    n_lhad += ok;
                } else {
                    ok = try_once<kMode, kBose>(cfg, p, u, pl, u_rap, n_viol);
                }
            } else {
                ok = try_any<kMode, kBose>(cfg, p, u, pl, u_rap, n_viol);
            }
            u.t++;
            u.tries_cell++;
            n_tries++;
            if (ok) {
                const int pid = pids[u.s];
                // the final cell of a redrawn hadron (cell_of then holds every
                // hadron's cell: the training rows of the learned proposal)
                if (u.redraw > 0 && u.phase == 0) cell_of[u.slot] = u.cell;
                if (kLcc)
                    emit_any<kMode>(cfg, cells, p, u.cell, u.phase ? -pid : pid, pl, u_rap, out,
                                    u.slot + u.phase);
                else
                    emit_any<kMode>(cfg, cells, p, u.cell, pid, pl, u_rap, out, u.slot);
                if (kLcc && u.mult == 2 && u.phase == 0) {
                    // the partner: same cell and mass, opposite B, S, Q
                    SpeciesDev sp2 = species[u.s];
                    sp2.baryon = -sp2.baryon;
                    sp2.strange = -sp2.strange;
                    sp2.charge = -sp2.charge;
                    u.phase = 1;
                    u.tries_cell = 0;
                    u.lp = nullptr;   // the pair's envelope is the hadron's, not the partner's
                    // (the lab-frame sampler keeps the hadron's maximum for
                    // its partner, src/emissionfunction.cpp:3503-3509)
                    if (!setup_any<kMode>(cfg, cells, sp2, u.cell, p, true, kBose)) {
                        atomicCAS(&ctrs->error_code, 0, 1);
                        ctrs->error_species = u.s;
                        write_hadron(out, u.slot + 1, 0, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f);
                        n_fail++;
                        active = false;
                    }
                } else {
                    active = false;
                }
            }
        }
    }
    // warp-aggregated counters
    unsigned long long w_tries = n_tries;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        w_tries += __shfl_down_sync(FULL, w_tries, o);
        n_redraws += __shfl_down_sync(FULL, n_redraws, o);
        n_fail += __shfl_down_sync(FULL, n_fail, o);
        n_viol += __shfl_down_sync(FULL, n_viol, o);
        if (kLearned) {
            n_ltries += __shfl_down_sync(FULL, n_ltries, o);
            n_lhad += __shfl_down_sync(FULL, n_lhad, o);
            lts.viol += __shfl_down_sync(FULL, lts.viol, o);
            lts.excess_tries += __shfl_down_sync(FULL, lts.excess_tries, o);
            lts.excess_hadrons += __shfl_down_sync(FULL, lts.excess_hadrons, o);
            lts.over_one += __shfl_down_sync(FULL, lts.over_one, o);
        }
    }
    if (lane == 0) {
        atomicAdd(&ctrs->tries, w_tries);
        if (n_redraws) atomicAdd(&ctrs->redraws, static_cast<unsigned long long>(n_redraws));
        if (n_fail) atomicAdd(&ctrs->failures, static_cast<unsigned long long>(n_fail));
        if (n_viol) atomicAdd(&ctrs->bound_violations, static_cast<unsigned long long>(n_viol));
        if (kLearned) {
            if (n_ltries) atomicAdd(&ctrs->learned_tries, static_cast<unsigned long long>(n_ltries));
            if (lts.viol) atomicAdd(&ctrs->learned_violations, static_cast<unsigned long long>(lts.viol));
            if (lts.excess_tries)
                atomicAdd(&ctrs->learned_excess_tries, static_cast<unsigned long long>(lts.excess_tries));
            if (lts.excess_hadrons)
                atomicAdd(&ctrs->learned_excess_hadrons,
                          static_cast<unsigned long long>(lts.excess_hadrons));
            if (lts.over_one)
                atomicAdd(&ctrs->learned_over_one, static_cast<unsigned long long>(lts.over_one));
            if (n_lhad) atomicAdd(&ctrs->learned_hadrons, static_cast<unsigned long long>(n_lhad));
        }
    }
}

// ---------------------------------------------------------------------------
// Learned proposal: network inputs, per-pair mixture records, envelope
// constants, and training rows from sampled hadrons.

// the 18 conditioning features of a (cell, species) pair (order and scales
// as declared in iss_gpu.h)
__device__ __forceinline__ void pair_features(const float4* __restrict__ rec, const SpeciesDev& sp,
                                              float (&f)[18]) {
    const float4 da = __ldg(rec + 1), th = __ldg(rec + 3), th2 = __ldg(rec + 4);
    const float4 pi1 = __ldg(rec + 5), pi2 = __ldg(rec + 6);
    const float T = th.x;
    const float m = sp.m_hi + sp.m_lo;
    const float mu = fminf(m, static_cast<float>(sp.baryon) * th.y + static_cast<float>(sp.strange) * th.z +
                                  static_cast<float>(sp.charge) * th.w);
    const float iep = 1.0f / (th2.x + th2.y);
    f[0] = (T - 0.15f) * 50.0f;
    f[1] = 0.5f * mu / T;
    f[2] = pi1.x * iep * 10.0f;
    f[3] = pi1.y * iep * 10.0f;
    f[4] = pi1.z * iep * 10.0f;
    f[5] = pi1.w * iep * 10.0f;
    f[6] = pi2.x * iep * 10.0f;
    f[7] = th2.w * iep * 20.0f;
    f[8] = 0.0f;
    f[9] = pi2.y * iep * 10.0f;
    f[10] = pi2.z * iep * 10.0f;
    f[11] = pi2.w * iep * 10.0f;
    const float D = sqrtf(da.y * da.y + da.z * da.z + da.w * da.w);
    const float nrm = fabsf(da.x) + D;
    const float inrm = nrm > 0.0f ? 1.0f / nrm : 0.0f;
    f[12] = da.x * inrm;
    f[13] = da.y * inrm;
    f[14] = da.z * inrm;
    f[15] = da.w * inrm;
    f[16] = 0.1f * m / T;
    f[17] = static_cast<float>(sp.sign);
}

__device__ __forceinline__ void store_features(const float (&f)[18], __nv_bfloat16* __restrict__ x) {
    uint4 w[4];
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(w);
#pragma unroll
    for (int j = 0; j < 16; j++) {
        const float a = 2 * j < 18 ? f[2 * j < 18 ? 2 * j : 0] : 0.0f;
        const float b = 2 * j + 1 < 18 ? f[2 * j + 1 < 18 ? 2 * j + 1 : 0] : 0.0f;
        h[j] = __floats2bfloat162_rn(a, b);
    }
    uint4* o = reinterpret_cast<uint4*>(x);
#pragma unroll
    for (int j = 0; j < 4; j++) o[j] = w[j];
}

// network input of pair (slot, cell) = slot * n_cells + cell
__global__ void learned_pair_features_kernel(CellArrays cells, const SpeciesDev* __restrict__ species,
                                             const int32_t* __restrict__ lspecies, int64_t n_cells,
                                             int64_t n_pairs, __nv_bfloat16* __restrict__ x) {
    const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (q >= n_pairs) return;
    const int slot = static_cast<int>(q / n_cells);
    const int64_t l = q - slot * n_cells;
    float f[18];
    pair_features(cells.rec + 8 * l, species[lspecies[slot]], f);
    store_features(f, x + q * 32);
}

constexpr int kEnvThreads = 128;

// envelope constant M of every pair: safety x the largest ratio
// P a / (alpha Q + (1 - alpha) P) over n_pilot proposals from q (Philox
// counter (draw, pair low, pair high, tag)), capped by the bound 1/(1 - alpha)
// that holds for every Q >= 0
__global__ void learned_pair_envelope_kernel(DevConfig cfg, CellArrays cells,
                                             const SpeciesDev* __restrict__ species,
                                             const int32_t* __restrict__ lspecies, int64_t n_cells,
                                             int64_t n_pairs, int n_pilot, float safety,
                                             float* __restrict__ lpairs) {
    // the block's records, staged once: every pilot proposal reads its
    // pair's record twice (component draw and density)
    // (a row stride of 17 float4: the lanes of a warp reading float4 j of
    // their own records hit distinct banks)
    constexpr int kRow = kPairFloats / 4 + 1;
    __shared__ float4 s_rec[kEnvThreads * kRow];
    const int64_t q0 = static_cast<int64_t>(blockIdx.x) * kEnvThreads;
    const int64_t nq = min(static_cast<int64_t>(kEnvThreads), n_pairs - q0);
    {
        const float4* src = reinterpret_cast<const float4*>(lpairs + q0 * kPairFloats);
        for (int i = threadIdx.x; i < nq * (kPairFloats / 4); i += kEnvThreads)
            s_rec[(i / (kPairFloats / 4)) * kRow + i % (kPairFloats / 4)] = src[i];
    }
    __syncthreads();
    const int64_t q = q0 + threadIdx.x;
    if (q >= n_pairs) return;
    const int slot = static_cast<int>(q / n_cells);
    const int64_t l = q - slot * n_cells;
    const float* lp = reinterpret_cast<const float*>(s_rec + threadIdx.x * kRow);
    const float cap = 1.0f / (1.0f - cfg.lalpha);
    Prop p;
    const float4 da = __ldg(cells.rec + 8 * l + 1);
    float best = 0.0f;
    if (da.x >= 0.0f && setup_prop(cfg, cells, species[lspecies[slot]], static_cast<int>(l), p)) {
        for (int j = 0; j < n_pilot; j++) {
            const uint32_t c3 = static_cast<uint32_t>(q >> 32) | (kTagPilot << 16);
            const uint4 A = block(2u * j, static_cast<uint32_t>(q), 0u, c3, cfg.key0, cfg.key1);
            const uint4 B = block(2u * j + 1u, static_cast<uint32_t>(q), 0u, c3, cfg.key0, cfg.key1);
            float K, nx, ny, nz, P, a;
            float4 pl;
            if (!propose_mixture<true>(p, lp, u01f(A.x) < cfg.lalpha, A, B, K, nx, ny, nz)) continue;
            if (!plain_target(cfg, p, K, nx, ny, nz, P, a, pl)) continue;
            const float Q = learned_density<true>(lp, K, nx, ny, nz);
            const float r = P * a / (cfg.lalpha * Q + (1.0f - cfg.lalpha) * P);
            if (r > best) best = r;
        }
    }
    lpairs[q * kPairFloats + 56] = best > 0.0f ? fminf(safety * best, cap) : cap;
}

// training rows from sampled hadrons: the pair's features and the rest-frame
// target (K, n); the species from the PDG id (sorted_pid / sorted_idx), the
// cell from cell_of.  Rows whose id is not a sampled species get K = 0 and
// are skipped by the host.
__device__ __forceinline__ void learned_train_row(
    const DevConfig& cfg, const CellArrays& cells, const SpeciesDev* __restrict__ species,
    const int32_t* __restrict__ sorted_pid, const int32_t* __restrict__ sorted_idx, int S,
    const HadronRec* __restrict__ had, const int32_t* __restrict__ cell_of, int64_t n,
    __nv_bfloat16* __restrict__ x, float4* __restrict__ tg, int64_t i, float& nll) {
    if (i >= n) return;
    const HadronRec h = had[i];
    int lo = 0, hi = S - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (sorted_pid[mid] < h.pid) lo = mid + 1; else hi = mid;
    }
    float f[18];
    if (S == 0 || sorted_pid[lo] != h.pid) {
        for (int j = 0; j < 18; j++) f[j] = 0.0f;
        store_features(f, x + i * 32);
        tg[i] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        return;
    }
    const SpeciesDev sp = species[sorted_idx[lo]];
    const int64_t l = cell_of[i];
    const float4* rec = cells.rec + 8 * l;
    pair_features(rec, sp, f);
    store_features(f, x + i * 32);
    const float4 u = __ldg(rec + 2), pos = __ldg(rec), th = __ldg(rec + 3);
    const float m = sp.m_hi + sp.m_lo;
    float E = h.E, pz = h.pz;
    if (cfg.hydro_mode != 2) {
        // boost-invariant records carry a drawn rapidity: back to the cell's frame
        const float mT = sqrtf(m * m + h.px * h.px + h.py * h.py);
        const float y = asinhf(h.pz / mT) - atanhf(h.z / h.t) + pos.w;
        E = mT * coshf(y);
        pz = mT * sinhf(y);
    }
    const float udp = u.y * h.px + u.z * h.py + u.w * pz;
    const float c = E - udp / (u.x + 1.0f);
    const float px = h.px - c * u.y, py = h.py - c * u.z, pzr = pz - c * u.w;
    const float p2 = px * px + py * py + pzr * pzr;
    const float pm = sqrtf(p2);
    const float K = p2 / (sqrtf(m * m + p2) + m) / th.x;
    const float ip = pm > 0.0f ? 1.0f / pm : 0.0f;
    tg[i] = make_float4(K, px * ip, py * ip, pzr * ip);
    Prop p;
    float P, a;
    float4 pl;
    if (setup_prop(cfg, cells, sp, static_cast<int>(l), p) &&
        plain_target(cfg, p, K, px * ip, py * ip, pzr * ip, P, a, pl) && P > 0.0f)
        nll = -logf(P);
}

__global__ void learned_train_rows_kernel(DevConfig cfg, CellArrays cells,
                                          const SpeciesDev* __restrict__ species,
                                          const int32_t* __restrict__ sorted_pid,
                                          const int32_t* __restrict__ sorted_idx, int S,
                                          const HadronRec* __restrict__ had,
                                          const int32_t* __restrict__ cell_of, int64_t n,
                                          __nv_bfloat16* __restrict__ x, float4* __restrict__ tg,
                                          double* __restrict__ nll_plain) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    float nll = 0.0f;
    learned_train_row(cfg, cells, species, sorted_pid, sorted_idx, S, had, cell_of, n, x, tg, i, nll);
    // the plain proposal's negative log-likelihood of the rows (the network's
    // loss on the same rows measures what it gains over the plain proposal)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nll += __shfl_xor_sync(0xffffffffu, nll, o);
    if ((threadIdx.x & 31) == 0 && nll != 0.0f) atomicAdd(nll_plain, static_cast<double>(nll));
}

}  // namespace

cudaError_t launch_counts(const DevConfig& cfg, const SpeciesDev* species, const double* totals,
                          double* pois, int32_t* counts, int32_t* items, int* error,
                          cudaStream_t stream) {
    const int64_t total = static_cast<int64_t>(cfg.n_events) * cfg.n_species;
    if (total <= 0) return cudaSuccess;
    const int rows = cfg.n_surfaces * cfg.n_species;
    PoissonC* pc = reinterpret_cast<PoissonC*>(pois);
    PoissonInv* inv = reinterpret_cast<PoissonInv*>(pc + rows);
    count_consts_kernel<<<(rows + 127) / 128, 128, 0, stream>>>(cfg, totals, pc, inv);
    const unsigned blocks = static_cast<unsigned>((total + 255) / 256);
    counts_kernel<<<blocks, 256, 0, stream>>>(cfg, species, totals, pc, inv, counts, items, error);
    return cudaGetLastError();
}

int offsets_num_tiles(int64_t n) { return static_cast<int>((n + kOffTile - 1) / kOffTile); }

cudaError_t launch_offsets_scan(const int32_t* counts, int64_t n, int64_t* tile_sum,
                                int64_t* offsets, cudaStream_t stream) {
    const int nt = offsets_num_tiles(n);
    if (nt == 0) return cudaMemsetAsync(offsets, 0, sizeof(int64_t), stream);
    off_tile_sum_kernel<<<nt, kOffThreads, 0, stream>>>(counts, n, tile_sum);
    off_tile_offset_kernel<<<1, kOffThreads, 0, stream>>>(tile_sum, nt, offsets, n);
    off_tile_scan_kernel<<<nt, kOffThreads, 0, stream>>>(counts, n, tile_sum, offsets);
    return cudaGetLastError();
}

cudaError_t launch_item_map(const int32_t* items, const int64_t* item_off, int64_t nseg,
                            int32_t* item_seg, cudaStream_t stream, const int64_t* limits) {
    if (nseg <= 0) return cudaSuccess;
    item_map_kernel<<<static_cast<unsigned>((nseg + 255) / 256), 256, 0, stream>>>(
        items, item_off, nseg, item_seg, limits);
    return cudaGetLastError();
}

cudaError_t launch_graph_limits(const int64_t* offsets, const int64_t* item_off, int64_t nseg,
                                int64_t cap_units, int64_t cap_items, int64_t* limits,
                                cudaStream_t stream) {
    graph_limits_kernel<<<1, 1, 0, stream>>>(offsets, item_off, nseg, cap_units, cap_items, limits);
    return cudaGetLastError();
}

cudaError_t launch_sampler(const DevConfig& cfg, const CellArrays& cells, const SpeciesDev* sp,
                           const int32_t* pids, const unsigned long long* cdf,
                           const int32_t* guide, const unsigned long long* qtot,
                           const int64_t* offsets,
                           const int64_t* item_off, const int32_t* item_seg, int64_t k_begin,
                           int64_t k_end, int32_t* cell_of, HadronRec* out,
                           unsigned long long* work_counter, SampleCounters* counters, int num_sms,
                           cudaStream_t stream, const int64_t* k_end_dev) {
    // with k_end_dev (graph replays) the item count is read on the device and
    // k_end is only the capacity that sizes the grids
    const int64_t n_items = k_end - k_begin;
    if (n_items <= 0) return cudaSuccess;
    {
        int64_t blocks = static_cast<int64_t>(num_sms) * std::max(1, cfg.assign_bps);
        const int64_t need = (n_items + (kAssignThreads / 32) - 1) / (kAssignThreads / 32);
        if (blocks > need) blocks = need;
        cell_assign_kernel<<<static_cast<unsigned>(blocks), kAssignThreads, 0, stream>>>(
            cfg, cdf, guide, qtot, offsets, item_off, item_seg, k_begin, k_end, sp, cell_of,
            k_end_dev);
    }
    const int per_sm = std::min(3, std::max(1, cfg.sampler_ctas));
    int64_t blocks = static_cast<int64_t>(num_sms) * per_sm;
    const int64_t max_blocks = (n_items + (kSampleThreads / 32) - 1) / (kSampleThreads / 32);
    if (blocks > max_blocks) blocks = max_blocks;
    if (blocks < 1) blocks = 1;
    const int mode = cfg.compat_fermion ? 0 : (cfg.include_diff ? 2 : 1);
    auto kernel =
        cfg.mc_sampling == 2
            ? (cfg.lcc ? sampler_kernel<true, false, 2, 0> : sampler_kernel<false, false, 2, 0>)
        : cfg.lpairs
            ? (mode == 1 ? (cfg.lcc ? sampler_kernel<true, true, 4, 1> : sampler_kernel<false, true, 4, 1>)
             : mode == 2 ? (cfg.lcc ? sampler_kernel<true, true, 4, 2> : sampler_kernel<false, true, 4, 2>)
                         : (cfg.lcc ? sampler_kernel<true, true, 4, 0> : sampler_kernel<false, true, 4, 0>))
        : mode == 1 ? (cfg.lcc ? sampler_kernel<true, false, 4, 1> : sampler_kernel<false, false, 4, 1>)
        : mode == 2 ? (cfg.lcc ? sampler_kernel<true, false, 4, 2> : sampler_kernel<false, false, 4, 2>)
                    : (cfg.lcc ? sampler_kernel<true, false, 4, 0> : sampler_kernel<false, false, 4, 0>);
    kernel<<<static_cast<unsigned>(blocks), kSampleThreads, 0, stream>>>(
        cfg, cells, sp, pids, cdf, guide, qtot, offsets, item_off, item_seg, k_begin,
        k_end, cell_of, out, work_counter, counters, k_end_dev);
    return cudaGetLastError();
}

cudaError_t launch_learned_pairs(const DevConfig& cfg, const CellArrays& cells,
                                 const SpeciesDev* species, const int32_t* lspecies, int n_slots,
                                 void* x, cudaStream_t stream) {
    const int64_t n_pairs = static_cast<int64_t>(n_slots) * cfg.n_cells;
    if (n_pairs <= 0) return cudaSuccess;
    learned_pair_features_kernel<<<static_cast<unsigned>((n_pairs + 255) / 256), 256, 0, stream>>>(
        cells, species, lspecies, cfg.n_cells, n_pairs, static_cast<__nv_bfloat16*>(x));
    return cudaGetLastError();
}

cudaError_t launch_learned_envelopes(const DevConfig& cfg, const CellArrays& cells,
                                     const SpeciesDev* species, const int32_t* lspecies, int n_slots,
                                     int n_pilot, float safety, float* lpairs, cudaStream_t stream) {
    const int64_t n_pairs = static_cast<int64_t>(n_slots) * cfg.n_cells;
    if (n_pairs <= 0) return cudaSuccess;
    learned_pair_envelope_kernel<<<static_cast<unsigned>((n_pairs + kEnvThreads - 1) / kEnvThreads),
                                   kEnvThreads, 0, stream>>>(
        cfg, cells, species, lspecies, cfg.n_cells, n_pairs, n_pilot, safety, lpairs);
    return cudaGetLastError();
}

cudaError_t launch_learned_train_rows(const DevConfig& cfg, const CellArrays& cells,
                                      const SpeciesDev* species, const int32_t* sorted_pid,
                                      const int32_t* sorted_idx, int S, const HadronRec* had,
                                      const int32_t* cell_of, int64_t n, void* x, void* tg,
                                      double* nll_plain, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    learned_train_rows_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(
        cfg, cells, species, sorted_pid, sorted_idx, S, had, cell_of, n,
        static_cast<__nv_bfloat16*>(x), static_cast<float4*>(tg), nll_plain);
    return cudaGetLastError();
}

}  // namespace iss
