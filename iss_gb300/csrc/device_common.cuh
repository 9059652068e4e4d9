// Device-side building blocks shared by the sampler kernels: the structures
// the kernels read, the Philox4x32-10 counter-based generator, uniform
// conversions and double-float ("float-float") helpers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace iss {

// ---------------------------------------------------------------------------
// structures passed to kernels by value

struct DevTables {
    const float4* sfK;      // [kSfLen] (K1, K2, K3, 0) in FP32, grid x = 0.5 + 0.05 i
    const float* sfE;       // [kSfLen * 9] E_2, E_4, ..., E_18 in FP32
    const double* b14c0;    // OSU 14-moment tables [iT * nmu + imu]
    const double* b14c1;
    const double* b14c2;
    int b14_nT, b14_nmu;
    double b14_T0, b14_mu0, b14_dT, b14_dmu;
    const double* ce;       // NEoS-BQS Chapman-Enskog, 200 * 200 rows of 5
    const double* qmu;      // RTA diffusion coefficient, 150 * 100
    const double* logfact;  // [kLogFactLen] log(k!) from the C library's lgamma
};

constexpr int kLogFactLen = 256;
constexpr int kPoissonConsts = 8;   // doubles per species, see poisson_consts
constexpr int kInvTable = 127;      // inversion CDF entries per species (+ length: 128 doubles)

// One surface of a batch.  The cells of all surfaces are concatenated; the
// per-(surface, species) rows of the cell CDF and of the guide tables are
// laid out surface by surface, species by species.
struct SurfSeg {
    int64_t c0, n;            // first cell, number of cells
    int64_t cdf_base;         // row (b, k) of the CDF starts at cdf_base + k (n + 1)
    int64_t guide_base;       // row (b, k) of the guide starts at guide_base + k (2^g + 1)
    int64_t tile_base;        // first flattened scan tile of the surface (S nt tiles)
    int nt, L, g;             // tiles per row, ceil(log2 n), guide bits
    int e0, ne;               // first event (batch numbering) and number of events
};

struct DevConfig {
    int hydro_mode;
    int include_shear, include_bulk, include_diff;
    int bulk_kind, neos_kind;
    int compat_fermion;
    int lcc;                 // local_charge_conservation (src/FSSW.cpp:931-938, 1035-1048)
    int sampling_model;
    double sampling_para1;
    float y_lb, y_rb;
    double ymult;            // y_RB - y_LB for boost-invariant surfaces, else 1
    uint32_t key0, key1;     // Philox key (the seed)
    int n_species;
    int n_events;
    int64_t n_cells;
    uint32_t event_offset;
    int max_tries, max_redraws;
    int chunk_events;        // events per sampling chunk (work-item order, see item_index)
    int n_surfaces;          // surfaces in the batch (1 for a single surface)
    const SurfSeg* surf;     // [n_surfaces]
    const int32_t* ev_surf;  // [n_events] surface of each event
    DevTables tab;
    // learned proposal (gpu_sampler = 1): slot of each species in the pair
    // tables (-1: plain proposal), the per-(slot, cell) mixture records of
    // kPairFloats floats, and the mixture weight of the network component
    const int32_t* lslot;
    const float* lpairs;
    float lalpha;
    // 1: exact rejection (the mixture with an excess branch, try_learned);
    // 0: the pilot envelope alone, whose ratios above 1 are counted
    int lexact;
    // launch shape (results do not depend on it; the autotuner picks it)
    int item_size;       // draws per sampler work item (multiple of 32, <= 1024)
    int yield_groups;    // species groups per cell in the yields kernel (grid y)
    // yields kernel: n_ygroups + 1 group starts, then the species of each
    // group (species with the same thermal series, yield_group_order)
    const int32_t* yorder;
    int n_ygroups;
    int sampler_ctas;    // sampler CTAs per SM (1..3)
    int assign_bps;      // cell-assignment blocks per SM
    // graph replays: (key0, key1, event_offset) of the call in device memory,
    // so one captured graph serves every seed; null: the fields above
    const uint32_t* run;
    // MC_sampling = 2 (EmissionFunctionArray, src/emissionfunction.cpp:3273-3623,
    // 4188-4421): pT sampled up to pt_max, y - eta_s in [-yme_range, yme_range],
    // delta f restricted to df_max_ratio of f0 when restrict_df
    int mc_sampling;         // 4: the FSSW sampler; 2: the lab-frame sampler
    float pt_max, yme_range, df_max_ratio;
    int restrict_df;
    // streamed generates: the record buffer and cell_of hold one chunk, whose
    // first record has the global slot slot_base (0 otherwise)
    int64_t slot_base;
};

// floats per (species slot, cell) record of the learned proposal: for each of
// the 8 mixture components (cumulative weight, log-normaliser c, mu, sigma,
// v_x, v_y, v_z, |v|); the last component's cumulative weight (always 1) is
// replaced by the envelope constant M of the pair
constexpr int kPairFloats = 64;

// Species record in the sampler's mass order (32 bytes).
struct SpeciesDev {
    float m_hi, m_lo;        // FP64 mass as a float-float pair
    float degen;             // spin degeneracy
    int light;               // mass < 0.7 GeV: 10 series terms (src/FSSW.cpp:740-745)
    int baryon, strange, charge, sign;
};

// Local-rest-frame cells, structure of arrays of float4.
struct CellArrays {
    float4* pos;    // tau, x, y, eta
    float4* da;     // dsigma_mu in the LRF (lower index); da.x < 0: cell dropped
    float4* u;      // u^mu in the t-z frame
    float4* th;     // T, muB, muS, muQ
    float4* th2;    // E, P, n_B, Pi
    float4* pi1;    // pi_xx, pi_xy, pi_xz, pi_yy (LRF)
    float4* pi2;    // pi_yz, q_x, q_y, q_z (LRF)
    float4* coef;   // per-cell delta-f coefficients vis0, vis1, vis2, kappa_B
    // the same eight float4 per cell as one 128-byte record (pos, da, u, th,
    // th2, pi1, pi2, coef): the sampler reads a random cell's record as one
    // cache line instead of eight
    float4* rec;
    // the lean FSSW sampler's constants of each cell, eight float4 (128
    // bytes) computed once by the prologue from the record above:
    // (t, x, y, z) for 3+1D surfaces, else (tau, x, y, eta); u^mu;
    // (d0, D, einv, T) and (n_x, n_y, n_z, 1/T) of the flux frame
    // dsigma_LRF = (d0, D n) with einv = 1/|t x n| (prop_e1);
    // (mu_B, mu_S, mu_Q, n_B/(e+P)); pi_xx, pi_xy, pi_xz, pi_yy times the
    // shear prefactor; (pi_yz times it, bulk b0 / m^2, b1 (/ B for kind 11),
    // b2); (bulk bi0 / m^2, q_x, q_y, q_z over kappa_B)
    float4* srec;
    // MC_sampling = 2 only (else null): the regulated Milne-frame cell, six
    // float4 per cell: (da0..da3), (u0..u3), (pi00 pi01 pi02 pi03),
    // (pi11 pi12 pi13 pi22), (pi23 pi33 q0 q1), (q2 q3 bulkPi 0)
    float4* milne;
};

// Resonance decay table (particle_decay::read_resonances_list): particles
// in pdg-file order with their channels; daughters are particle indices.
struct DecayParticle {
    int32_t pid;
    float mass, width;
    int32_t stable;
    int32_t first_channel, n_channels;
};
struct DecayChannel {
    int32_t n_daughters;
    double branching_ratio;
    int32_t daughter[5];
    // ceil(2^53 x the FP64 sum of the branching ratios of this and the
    // particle's earlier channels, summed in channel order): a 53-bit uniform
    // m 2^-53 lies below that sum exactly when m < cum53
    uint64_t cum53;
};
struct DecayTablesDev {
    const DecayParticle* particles;
    const DecayChannel* channels;
    const int32_t* sorted_pid;   // pids in increasing order ...
    const int32_t* sorted_idx;   // ... and their particle indices
    int n_particles;
    // open-addressing table pid -> particle index: kDecayHash (pid, index)
    // pairs, linear probing from decay_hash(pid), pid 0 marks an empty slot
    const int2* hash;
};
constexpr int kDecayHash = 2048;
__host__ __device__ inline uint32_t decay_hash(int32_t pid) {
    return (static_cast<uint32_t>(pid) * 2654435761u) >> 21;   // 11 bits: kDecayHash slots
}

// Counters written by the sampler.
struct SampleCounters {
    unsigned long long tries;
    unsigned long long redraws;
    unsigned long long failures;
    unsigned long long bound_violations;
    unsigned long long learned_tries;       // proposals of the learned sampler
    unsigned long long learned_violations;  // of these, ratios above the envelope M
    unsigned long long learned_hadrons;     // hadrons of species in the pair tables
    unsigned long long learned_excess_tries;    // exact mode: proposals of the excess branch
    unsigned long long learned_excess_hadrons;  // exact mode: hadrons accepted there
    unsigned long long learned_over_one;        // exact mode: mixture-branch ratios above 1
    int error_code;          // 1: m/T - mu/T off the momentum tables
    int error_species;
};

// Hadron record, layout of iSS_Hadron / iss_hadron_t.
struct HadronRec {
    int pid;
    float mass, E, px, py, pz, t, x, y, z;
};

enum : uint32_t { kTagCell = 1u, kTagTry = 2u, kTagCount = 3u, kTagLearn = 5u, kTagPilot = 6u,
                  kTagLearnRap = 7u, kTagEfa = 8u, kTagEfaRap = 9u };

// ---------------------------------------------------------------------------
// Fixed-point cell CDF.
//
// The reference draws a cell by a binary search in the FP64 running sum of
// the per-cell yields (RandomVariable1DArray, src/RandomVariable1DArray.cpp:25-74,
// used at src/FSSW.cpp:1003-1006).  Here every FP32 yield y of species s is
// truncated to the integer q = floor(y * 2^E_s), with E_s chosen from the
// species' largest yield and the cell count so that the sum Q_s of all q
// stays below 2^62.  Integer prefix sums are exact in any order: the tiles of
// the scan need no particular order, and a CPU replay gets the same bits.
// A cell is drawn from 64 random bits r: v = floor(r * Q_s / 2^64) is uniform
// on [0, Q_s), and the cell is the i with C[i] <= v < C[i+1].  Cells whose
// q is 0 are never drawn, as cells of zero yield are never drawn in the
// reference.  The per-species total yield is Q_s * 2^-E_s.
#if defined(__CUDACC__)
#define ISS_HD __host__ __device__
#else
#define ISS_HD
#endif

// ceil(log2 n), 0 for n <= 1
ISS_HD inline int cdf_log2_cells(int64_t n) {
    int L = 0;
    while (L < 62 && (int64_t(1) << L) < n) ++L;
    return L;
}

// 2^g guide buckets per row, g = clamp(ceil(log2 n) - 1, 1, 24): between n/2
// and n buckets, so a bucket spans one or two cells on average
ISS_HD inline int cdf_guide_bits(int64_t n) {
    const int g = cdf_log2_cells(n) - 1;
    return g < 1 ? 1 : (g > 24 ? 24 : g);
}

// q(y) = mantissa(y) * 2^(exponent(y) + base) with base = 38 - L - e_max,
// e_max the biased exponent of the species' largest yield; E_s = 150 + base.
// Every q is below 2^(62 - L), so the sum over at most 2^L cells is below 2^62.
ISS_HD inline int cdf_quant_base(uint32_t ymax_bits, int L) {
    int ex = static_cast<int>((ymax_bits >> 23) & 0xFFu);
    if (ex == 0) ex = 1;
    return 38 - L - ex;
}

ISS_HD inline uint64_t cdf_quantize(uint32_t y_bits, int base) {
    int e = static_cast<int>((y_bits >> 23) & 0xFFu);
    uint32_t m = y_bits & 0x7FFFFFu;
    if (e) m |= 0x800000u; else e = 1;
    const int sh = e + base;
    if (sh >= 0) return static_cast<uint64_t>(m) << sh;
    if (sh <= -24) return 0;
    return static_cast<uint64_t>(m >> (-sh));
}

#if defined(__CUDACC__)
// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z);
        const uint32_t lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// [0, 1), 23 bits: the top 23 bits as the mantissa of a float in [1, 2),
// minus 1 (exact; no integer-to-float conversion)
__device__ __forceinline__ float u01f(uint32_t x) {
    return __uint_as_float((x >> 9) | 0x3F800000u) - 1.0f;
}
// (0, 1], 23 bits: 2 minus the same float in [1, 2) (exact, never 0)
__device__ __forceinline__ float u01f_pos(uint32_t x) {
    return 2.0f - __uint_as_float((x >> 9) | 0x3F800000u);
}
// [0, 1), 53 bits
__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
    // (a >> 5) * 2^26 + (b >> 6) is an integer below 2^53: converted exactly
    const unsigned long long m =
        (static_cast<unsigned long long>(a >> 5) << 26) | static_cast<unsigned long long>(b >> 6);
    return static_cast<double>(m) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------------------
// float-float arithmetic (error-free transformations)

__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
    p = a * b;
    e = fmaf(a, b, -p);
}
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }

// the configuration with the call's seed and event offset (DevConfig::run)
__device__ __forceinline__ DevConfig with_run_keys(const DevConfig& c) {
    DevConfig r = c;
    if (c.run) {
        r.key0 = c.run[0];
        r.key1 = c.run[1];
        r.event_offset = c.run[2];
    }
    return r;
}
#endif  // __CUDACC__

}  // namespace iss
