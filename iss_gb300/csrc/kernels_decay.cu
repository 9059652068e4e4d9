// Resonance decays of the sampled hadrons (FSSW::perform_resonance_feed_down,
// src/FSSW.cpp:1746-1779, with particle_decay::perform_decays and the two-
// and three-body kinematics of src/particle_decay.cpp:265-513).
//
// The reference walks each event's list: a stable hadron goes to the output,
// an unstable one decays and its daughters go to the output (stable) or to
// the end of the list (unstable).  The output of an event is therefore, in
// order, the stable products of the sampled hadrons, then those of their
// unstable daughters, then of the granddaughters, and so on.  Here each such
// generation is one pass over all events at once, in two sweeps.
//
// The count sweep runs the generations on particle ids alone: a hadron's
// channel and the kinds of its products do not depend on momenta.  Per
// generation a count kernel (channel choice; stable and unstable products per
// hadron) and one packed exclusive scan, which also writes the ids and events
// of the unstable products (the next generation's input), give the sizes of
// every generation and, per event, its range of inputs and its number of
// stable products.  That fixes each event's final list, and the place of
// every generation's stable products in it, before any kinematics run.
//
// The write sweep runs the generations again with momenta: stable inputs are
// copied and decaying ones decay, their stable products going straight to
// their final places and the unstable ones to the next generation's records.
//
// The sizes live on the device (DecayMeta): each count-sweep kernel reads its
// input size there, so the host enqueues batches of generations without
// waiting.  A generation whose products would not fit a buffer raises a flag
// and ends the chain before the write sweep; the host then reruns the count
// sweep with larger buffers (the results do not depend on the buffer sizes).
//
// Every random number comes from Philox4x32-10 with counter
// (draw, index of the hadron in its event's generation list, event,
// generation | kTagDecay << 16): results do not depend on thread mapping.
#include <cuda_runtime.h>

#include <algorithm>

#include "device_common.cuh"
#include "kernels.h"

namespace iss {

namespace {

constexpr int kDecayThreads = 256;
constexpr uint32_t kTagDecay = 4u;
constexpr int kThreeBodyTries = 100000;
// angles uniform on [-pi, pi), where the SFU's sine and cosine are accurate to 2^-20
constexpr float kTwoPiD = 6.2831853071795865f;

__device__ __forceinline__ uint4 dblock(uint32_t draw, uint32_t i, uint32_t e, uint32_t gen,
                                        uint32_t k0, uint32_t k1) {
    return philox4x32_10(make_uint4(draw, i, e, gen | (kTagDecay << 16)), k0, k1);
}

// particle index of pid from the hash table staged in shared memory, -1 if
// absent (bounded probe)
__device__ __forceinline__ int lookup_hash(const int2* __restrict__ h, int pid) {
    uint32_t j = decay_hash(pid);
    for (int k = 0; k < kDecayHash; k++, j = (j + 1) & (kDecayHash - 1)) {
        const int2 v = h[j];
        if (v.x == pid) return v.y;
        if (v.x == 0) return -1;
    }
    return -1;
}

// The channel of an unstable particle (cumulated branching ratios against one
// uniform, src/particle_decay.cpp:283-293), or -1 when the ratios do not
// reach the uniform.  The uniform is m 2^-53 (u53) and the FP64 partial sums
// are held as the integers cum53 = ceil(2^53 sum): sum > u exactly when
// m < cum53, so the choice equals the FP64 comparison without FP64 work.
__device__ __forceinline__ int pick_channel(const DecayTablesDev& t, int type, unsigned long long m) {
    const int c0 = t.particles[type].first_channel, nc = t.particles[type].n_channels;
    for (int c = 0; c < nc; c++) {
        if (m < t.channels[c0 + c].cum53) return c0 + c;
    }
    return -1;
}

__device__ __forceinline__ unsigned long long u53_bits(uint32_t a, uint32_t b) {
    return (static_cast<unsigned long long>(a >> 5) << 26) | static_cast<unsigned long long>(b >> 6);
}

struct DecayPlan {
    int type, channel, n;      // n: daughters (0: none written, 1: the particle itself)
};

__device__ DecayPlan plan(const DecayTablesDev& t, const int2* __restrict__ hash, const DevConfig& cfg,
                          int pid, uint32_t i, uint32_t eg, uint32_t gen) {
    DecayPlan d{};
    d.type = lookup_hash(hash, pid);
    d.channel = -1;
    if (d.type < 0 || t.particles[d.type].stable) {
        d.n = 1;
        return d;
    }
    const uint4 w = dblock(0u, i, eg, gen, cfg.key0, cfg.key1);
    d.channel = pick_channel(t, d.type, u53_bits(w.x, w.y));
    const int nd = d.channel >= 0 ? t.channels[d.channel].n_daughters : 0;
    // the reference decays into two or three bodies only; other channels
    // leave no product (src/particle_decay.cpp:294-330)
    d.n = (nd == 2 || nd == 3) ? nd : 0;
    return d;
}

__device__ __forceinline__ bool daughter_stable(const DecayTablesDev& t, int idx) {
    return idx < 0 || t.particles[idx].stable;
}

// one 40-byte record as five 8-byte words (records are 8-byte aligned)
__device__ __forceinline__ void copy_rec(HadronRec* __restrict__ dst, const HadronRec* __restrict__ src) {
    const uint2* s = reinterpret_cast<const uint2*>(src);
    uint2* d = reinterpret_cast<uint2*>(dst);
#pragma unroll
    for (int k = 0; k < 5; k++) d[k] = s[k];
}

// a record built in registers, stored as five 8-byte words
__device__ __forceinline__ void store_rec(HadronRec* __restrict__ dst, const HadronRec& r) {
    float2* d = reinterpret_cast<float2*>(dst);
    d[0] = make_float2(__int_as_float(r.pid), r.mass);
    d[1] = make_float2(r.E, r.px);
    d[2] = make_float2(r.py, r.pz);
    d[3] = make_float2(r.t, r.x);
    d[4] = make_float2(r.y, r.z);
}

// channel cache of a hadron: (particle type << 16) | decay channel (the host
// checks that both fit), or kChanStable (kept as it is) or kChanNone (no
// product: no channel reached the uniform, or a channel of other than two
// or three bodies)
constexpr int32_t kChanStable = -1;
constexpr int32_t kChanNone = -2;

__device__ __forceinline__ int64_t meta_n(const int64_t* __restrict__ meta, uint32_t gen) {
    return meta[kDecayMetaNIn + gen];
}
// where generation gen's inputs start in the per-input arrays (its scan
// starts at meta_ib + gen: each scan has one entry more than its inputs)
__device__ __forceinline__ int64_t meta_ib(const int64_t* __restrict__ meta, uint32_t gen) {
    return meta[kDecayMetaIBase + gen];
}

// Count kernel of generation gen: the channel cache and the packed counts of
// every input.  The particle id comes from the sampled records (generation 0)
// or from the ids the previous generation's scan wrote (later generations).
__global__ void __launch_bounds__(kDecayThreads)
decay_count_kernel(DevConfig cfg, DecayTablesDev t, uint32_t gen, const HadronRec* __restrict__ rec0,
                   const int32_t* __restrict__ pid_all, const int32_t* __restrict__ ev_all,
                   const int64_t* __restrict__ first, const int64_t* __restrict__ meta,
                   int32_t* __restrict__ chan_all, int64_t* __restrict__ cnt) {
    __shared__ int2 s_hash[kDecayHash];
    const int64_t n = meta_n(meta, gen), ib = meta_ib(meta, gen);
    // blocks without inputs leave before staging the table (late generations
    // are small)
    if (static_cast<int64_t>(blockIdx.x) * blockDim.x >= n) return;
    for (int j = threadIdx.x; j < kDecayHash; j += blockDim.x) s_hash[j] = t.hash[j];
    __syncthreads();
    const int32_t* ev = ev_all + ib;
    int32_t* chan = chan_all + ib;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int e = ev[i];
        const int pid = gen == 0 ? rec0[i].pid : pid_all[ib + i];
        const DecayPlan d = plan(t, s_hash, cfg, pid, static_cast<uint32_t>(i - first[e]),
                                 cfg.event_offset + static_cast<uint32_t>(e), gen);
        int s = 0, u = 0;
        int32_t c;
        if (d.channel < 0) {
            s = d.n;   // stable (or no channel: nothing)
            c = d.n == 1 ? kChanStable : kChanNone;
        } else if (d.n == 0) {
            c = kChanNone;
        } else {
            c = static_cast<int32_t>((static_cast<uint32_t>(d.type) << 16) |
                                     static_cast<uint32_t>(d.channel));
            for (int k = 0; k < d.n; k++) {
                if (daughter_stable(t, t.channels[d.channel].daughter[k])) s++; else u++;
            }
        }
        chan[i] = c;
        cnt[i] = (static_cast<int64_t>(s) << 32) | static_cast<int64_t>(u);
    }
}

// The mother's 4-velocity: gamma = E/m and u = p/m (computing gamma from
// 1 - v^2 in FP32 would lose digits for fast mothers)
struct Lorentz {
    float ux, uy, uz, gamma;
};

__device__ __forceinline__ Lorentz velocity(const HadronRec& m) {
    Lorentz L;
    const float inv = 1.0f / m.mass;
    L.ux = m.px * inv;
    L.uy = m.py * inv;
    L.uz = m.pz * inv;
    L.gamma = m.E * inv;
    return L;
}

// rest-frame (E, p) of a daughter boosted with the mother's velocity,
// the reference's p + ((gamma-1) v.p / v^2 + gamma E) v written with u:
// E' = gamma E + u.p,  p' = p + (E + u.p / (gamma + 1)) u
__device__ __forceinline__ void boost(const Lorentz& L, float E, float px, float py, float pz,
                                      float* oE, float* ox, float* oy, float* oz) {
    const float up = L.ux * px + L.uy * py + L.uz * pz;
    const float c = E + up / (L.gamma + 1.0f);
    *oE = L.gamma * E + up;
    *ox = px + c * L.ux;
    *oy = py + c * L.uy;
    *oz = pz + c * L.uz;
}

// the products of hadron *mp of event e (index ie in its event's
// generation list) through channel `channel` of particle `type`: stable ones
// from out_s[ps], unstable ones from out_u[pu].  The decay point and the
// mother's velocity come first, so that each daughter is boosted and stored
// as soon as its rest-frame momentum is known.
__device__ __noinline__ void decay_one(const DevConfig& cfg, const DecayTablesDev& t, uint32_t gen,
                                       const HadronRec* __restrict__ mp_rec, int e, uint32_t ie, int type,
                                       int channel, int64_t ps, int64_t pu, HadronRec* __restrict__ out_s,
                                       HadronRec* __restrict__ out_u,
                                       unsigned long long* __restrict__ failures) {
    const uint32_t eg = cfg.event_offset + static_cast<uint32_t>(e);
    const DecayChannel& ch = t.channels[channel];
    const int n = ch.n_daughters;
    const DecayParticle& mp = t.particles[type];
    const float M = mp.mass;       // pole mass (the reference does not sample Breit-Wigner)
    float md[3];
    for (int k = 0; k < n; k++) {
        const int di = ch.daughter[k];
        md[k] = di >= 0 ? t.particles[di].mass : 0.0f;
    }
    const uint4 w1 = dblock(1u, ie, eg, gen, cfg.key0, cfg.key1);
    float dt, dx, dy, dz;
    Lorentz L;
    {
        const HadronRec m = *mp_rec;
        // life time gamma / Gamma in fm (src/particle_decay.cpp:396-401)
        float life = 1e10f;
        if (mp.width > 1e-10f) {
            const float tau0 = m.E / M / mp.width;
            life = -tau0 * __logf(u01f_pos(w1.w)) * 0.19733f;
        }
        const float inv = 1.0f / m.E;
        dt = m.t + life;
        dx = m.x + m.px * inv * life;
        dy = m.y + m.py * inv * life;
        dz = m.z + m.pz * inv * life;
        L = velocity(m);
    }
    auto emit = [&](int k, float E, float px, float py, float pz) {
        HadronRec r;
        const int di = ch.daughter[k];
        r.pid = di >= 0 ? t.particles[di].pid : 0;
        r.mass = md[k];
        boost(L, E, px, py, pz, &r.E, &r.px, &r.py, &r.pz);
        r.t = dt;
        r.x = dx;
        r.y = dy;
        r.z = dz;
        if (daughter_stable(t, di)) {
            store_rec(out_s + ps, r);
            ps++;
        } else {
            store_rec(out_u + pu, r);
            pu++;
        }
    };
    if (n == 2) {
        const float m1 = md[0], m2 = md[1];
        const float a = M * M - m1 * m1 - m2 * m2;
        const float p = sqrtf(fmaxf(a * a - 4.0f * m1 * m1 * m2 * m2, 0.0f)) / (2.0f * M);
        float sphi, cphi;
        __sincosf(kTwoPiD * (u01f(w1.x) - 0.5f), &sphi, &cphi);
        const float cth = 2.0f * (u01f(w1.y) - 0.5f);
        const float sth = sqrtf(fmaxf(1.0f - cth * cth, 0.0f));
        const float px = p * sth * cphi, py = p * sth * sphi, pz = p * cth;
        emit(0, sqrtf(p * p + m1 * m1), px, py, pz);
        emit(1, sqrtf(p * p + m2 * m2), -px, -py, -pz);
    } else {
        // phase space by rejection on (E1, E2) (src/particle_decay.cpp:445-458)
        const float m1 = md[0], m2 = md[1], m3 = md[2];
        const float span = M - m1 - m2 - m3;
        float E1 = m1, E2 = m2, p1 = 0.f, p2 = 0.f, c12 = 0.f;
        bool ok = false;
        // two (E1, E2) candidates per Philox block: (x, y), then (z, w)
        for (int it = 0; it < kThreeBodyTries / 2 && !ok; it++) {
            const uint4 w = dblock(16u + static_cast<uint32_t>(it), ie, eg, gen, cfg.key0, cfg.key1);
#pragma unroll
            for (int h = 0; h < 2 && !ok; h++) {
                E1 = u01f(h ? w.z : w.x) * span + m1;
                E2 = u01f(h ? w.w : w.y) * span + m2;
                if (E1 + E2 > M) continue;
                p1 = sqrtf(fmaxf(E1 * E1 - m1 * m1, 0.0f));
                p2 = sqrtf(fmaxf(E2 * E2 - m2 * m2, 0.0f));
                const float E3 = M - E1 - E2;
                c12 = (E3 * E3 - p1 * p1 - p2 * p2 - m3 * m3) / (2.0f * p1 * p2);
                ok = (c12 >= -1.0f && c12 <= 1.0f);
            }
        }
        if (!ok) {
            atomicAdd(failures, 1ull);
            c12 = 1.0f;
        }
        const float tp2x = p2 * sqrtf(fmaxf(1.0f - c12 * c12, 0.0f)), tp2z = p2 * c12;
        const float tp3x = -tp2x, tp3z = -(p1 + tp2z);
        float sphi, cphi, sksi, cksi;
        __sincosf(kTwoPiD * (u01f(w1.x) - 0.5f), &sphi, &cphi);
        __sincosf(kTwoPiD * (u01f(w1.y) - 0.5f), &sksi, &cksi);
        const float cth = 2.0f * u01f(w1.z) - 1.0f;
        const float sth = sqrtf(fmaxf(1.0f - cth * cth, 0.0f));
        {
            const float px = -p1 * sth * cksi, py = p1 * sth * sksi, pz = p1 * cth;
            emit(0, sqrtf(md[0] * md[0] + px * px + py * py + pz * pz), px, py, pz);
        }
        {
            const float px = tp2x * (cphi * cth * cksi - sphi * sksi) - tp2z * sth * cksi;
            const float py = tp2x * (-cphi * cth * sksi - sphi * cksi) + tp2z * sth * sksi;
            const float pz = tp2x * (cphi * sth) + tp2z * cth;
            emit(1, sqrtf(md[1] * md[1] + px * px + py * py + pz * pz), px, py, pz);
        }
        {
            const float px = tp3x * (cphi * cth * cksi - sphi * sksi) - tp3z * sth * cksi;
            const float py = tp3x * (-cphi * cth * sksi - sphi * cksi) + tp3z * sth * sksi;
            const float pz = tp3x * cphi * sth + tp3z * cth;
            emit(2, sqrtf(md[2] * md[2] + px * px + py * py + pz * pz), px, py, pz);
        }
    }
}

// The write pass of a generation.  Each warp walks its chunks of 32 inputs:
// stable inputs are copied to their final places at once, decaying ones are
// queued in shared memory, and whenever 32 are queued the whole warp decays
// them together, so lanes that copy do not wait on lanes that decay.  Stable
// product k of input i (event e) goes to shift[e] + stable(off[i]) + k, where
// shift[e] is the final place of the event's first stable product of this
// generation less its scan offset; unstable ones to out_u[unstable(off[i])].
constexpr int kDecayQueue = 64;

__global__ void __launch_bounds__(kDecayThreads, 3)
decay_write_kernel(DevConfig cfg, DecayTablesDev t, uint32_t gen, int64_t n,
                   const HadronRec* __restrict__ in, const int32_t* __restrict__ ev,
                   const int64_t* __restrict__ first, const int32_t* __restrict__ chan,
                   const int64_t* __restrict__ off, const int64_t* __restrict__ shift,
                   HadronRec* __restrict__ out, HadronRec* __restrict__ out_u,
                   unsigned long long* __restrict__ failures) {
    __shared__ int64_t s_q[kDecayThreads / 32][kDecayQueue];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t* q = s_q[wid];
    int qn = 0;   // queued inputs (warp-uniform, < 32 between chunks)
    auto decay = [&](int64_t i) {
        const int32_t c = chan[i];
        const int e = ev[i];
        const int64_t o = off[i];
        decay_one(cfg, t, gen, in + i, e, static_cast<uint32_t>(i - first[e]), c >> 16, c & 0xFFFF,
                  shift[e] + (o >> 32), o & 0xFFFFFFFFll, out, out_u, failures);
    };
    const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
    for (int64_t b0 = (static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + wid) * 32; b0 < n;
         b0 += warps * 32) {
        const int64_t i = b0 + lane;
        const int32_t c = i < n ? chan[i] : kChanNone;
        if (c == kChanStable) copy_rec(out + shift[ev[i]] + (off[i] >> 32), in + i);
        const unsigned want = __ballot_sync(FULL, c >= 0);
        if (c >= 0) q[qn + __popc(want & ((1u << lane) - 1u))] = i;
        qn += __popc(want);
        __syncwarp();
        if (qn >= 32) {
            decay(q[lane]);
            __syncwarp();
            if (lane < qn - 32) q[lane] = q[32 + lane];
            __syncwarp();
            qn -= 32;
        }
    }
    if (lane < qn) decay(q[lane]);
}

// event ids of the sampled records from the event offsets
__global__ void event_ids_kernel(const int64_t* __restrict__ off, int n_events,
                                 int32_t* __restrict__ ev) {
    const int e = blockIdx.x;
    if (e >= n_events) return;
    for (int64_t i = off[e] + threadIdx.x; i < off[e + 1]; i += blockDim.x) ev[i] = e;
}

// generation 0's input range per event: the sampled records of the event
__global__ void dk_first_gen_kernel(const int64_t* __restrict__ evoff, int n_events,
                                    int64_t* __restrict__ first, int64_t* __restrict__ last) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_events) return;
    const bool any = evoff[e + 1] > evoff[e];
    first[e] = any ? evoff[e] : -1;
    last[e] = any ? evoff[e + 1] : -1;
}

// ---- exclusive scans of the packed counts, input size on the device ----

constexpr int kDkScanThreads = 256;
constexpr int kDkScanPer = 16;
constexpr int kDkTile = kDkScanThreads * kDkScanPer;

__device__ __forceinline__ long long dk_warp_incl(long long v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long x = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += x;
    }
    return v;
}

// block-wide exclusive scan of one value per thread; *total = the sum
__device__ long long dk_block_excl(long long v, long long* s_warp, long long* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const long long inc = dk_warp_incl(v);
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        const long long w = lane < nw ? s_warp[lane] : 0;
        const long long wi = dk_warp_incl(w);
        if (lane < nw) s_warp[lane] = wi - w;
        if (lane == nw - 1) s_warp[32] = wi;
    }
    __syncthreads();
    const long long out = s_warp[wid] + inc - v;
    *total = s_warp[32];
    __syncthreads();
    return out;
}

// Exclusive scan of the packed counts (stable << 32 | unstable): one int64
// scan gives both offsets, since no partial sum of the unstable half reaches
// 2^32 (it is bounded by the next-input capacity).  Generation gen's scan
// lands at off_all + meta_ib + gen (n + 1 entries, the last the total).
// tile sums: tiles[t] for the tiles of 4096 inputs
__global__ void __launch_bounds__(kDkScanThreads)
dk_tile_sum_kernel(const int64_t* __restrict__ c, const int64_t* __restrict__ meta, uint32_t gen,
                   int64_t* __restrict__ tiles) {
    __shared__ long long s_warp[33];
    const int64_t n = meta_n(meta, gen);
    const int64_t nt = (n + kDkTile - 1) / kDkTile;
    for (int64_t tl = blockIdx.x; tl < nt; tl += gridDim.x) {
        long long acc = 0;
        for (int k = 0; k < kDkScanPer; k++) {
            const int64_t i = tl * kDkTile + k * kDkScanThreads + threadIdx.x;
            if (i < n) acc += c[i];
        }
        long long tot;
        dk_block_excl(acc, s_warp, &tot);
        if (threadIdx.x == 0) tiles[tl] = tot;
    }
}

// one block: tile sums -> tile offsets (in place), the total to off[n]
__global__ void __launch_bounds__(kDkScanThreads)
dk_tile_offset_kernel(int64_t* __restrict__ tiles, const int64_t* __restrict__ meta, uint32_t gen,
                      int64_t* __restrict__ off_all) {
    __shared__ long long s_warp[33];
    const int64_t n = meta_n(meta, gen);
    const int64_t nt = (n + kDkTile - 1) / kDkTile;
    long long carry = 0;
    for (int64_t b0 = 0; b0 < nt; b0 += kDkScanThreads) {
        const int64_t i = b0 + threadIdx.x;
        const long long v = i < nt ? tiles[i] : 0;
        long long tot;
        const long long ex = dk_block_excl(v, s_warp, &tot);
        if (i < nt) tiles[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) off_all[meta_ib(meta, gen) + gen + n] = carry;
}

// the next generation's inputs made by input c (a decaying hadron of event
// e): the particle id and event of each unstable product, from slot pu on;
// slots at or past i_cap are skipped (the generation then fails the size
// check and the call reruns)
__device__ void write_daughters(const DecayTablesDev& t, int32_t c, int e, int64_t pu, int64_t i_cap,
                                int32_t* __restrict__ ev_all, int32_t* __restrict__ pid_all) {
    const DecayChannel& ch = t.channels[c & 0xFFFF];
    for (int k = 0; k < ch.n_daughters; k++) {
        const int di = ch.daughter[k];
        if (daughter_stable(t, di)) continue;
        if (pu < i_cap) {
            pid_all[pu] = t.particles[di].pid;
            ev_all[pu] = e;
        }
        pu++;
    }
}

// The scan of each tile, and the next generation's inputs: a thread scans 16
// consecutive inputs and writes the products of those with unstable ones
// (whose inputs follow this generation's, at meta_ib + n); the offsets go
// back through shared memory to coalesced stores.
__global__ void __launch_bounds__(kDkScanThreads)
dk_tile_scan_kernel(DecayTablesDev t, const int64_t* __restrict__ c, const int64_t* __restrict__ meta,
                    uint32_t gen, const int64_t* __restrict__ tiles, const int32_t* __restrict__ chan_all,
                    int32_t* __restrict__ ev_all, int32_t* __restrict__ pid_all, int64_t i_cap,
                    int64_t* __restrict__ off_all) {
    __shared__ long long s_in[kDkScanThreads * (kDkScanPer + 1)];
    __shared__ long long s_warp[33];
    const int64_t n = meta_n(meta, gen), ib = meta_ib(meta, gen), nb = ib + n;
    const int64_t nt = (n + kDkTile - 1) / kDkTile;
    int64_t* off = off_all + ib + gen;
    for (int64_t tl = blockIdx.x; tl < nt; tl += gridDim.x) {
        const int64_t t0 = tl * kDkTile;
        for (int k = 0; k < kDkScanPer; k++) {
            const int e = k * kDkScanThreads + threadIdx.x;
            const int64_t i = t0 + e;
            s_in[(e / kDkScanPer) * (kDkScanPer + 1) + e % kDkScanPer] = i < n ? c[i] : 0;
        }
        __syncthreads();
        long long* mine = s_in + threadIdx.x * (kDkScanPer + 1);
        long long acc = 0;
#pragma unroll
        for (int k = 0; k < kDkScanPer; k++) acc += mine[k];
        long long tot;
        long long run = tiles[tl] + dk_block_excl(acc, s_warp, &tot);
        const int64_t e0 = t0 + static_cast<int64_t>(threadIdx.x) * kDkScanPer;
        for (int k = 0; k < kDkScanPer; k++) {
            const long long v = mine[k];
            if ((v & 0xFFFFFFFFll) != 0)
                write_daughters(t, chan_all[ib + e0 + k], ev_all[ib + e0 + k], nb + (run & 0xFFFFFFFFll),
                                i_cap, ev_all, pid_all);
            mine[k] = run;
            run += v;
        }
        __syncthreads();
        for (int k = 0; k < kDkScanPer; k++) {
            const int e = k * kDkScanThreads + threadIdx.x;
            const int64_t i = t0 + e;
            if (i < n) off[i] = s_in[(e / kDkScanPer) * (kDkScanPer + 1) + e % kDkScanPer];
        }
        __syncthreads();
    }
}

// Sizes of the next generation: its inputs (this generation's unstable
// products) follow this generation's in the per-input arrays, and the stable
// products so far give the final lists' length.  A generation that does not
// fit (final lists, one generation's records, all inputs) or would exceed
// g_max sets a flag, records what it needed and ends the chain.
__global__ void dk_advance_kernel(int64_t* __restrict__ meta, uint32_t gen, const int64_t* __restrict__ off_all,
                                  int64_t s_cap, int64_t u_cap, int64_t i_cap, uint32_t g_max) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int64_t n = meta[kDecayMetaNIn + gen];
    const int64_t ib = meta[kDecayMetaIBase + gen];
    const int64_t sb = meta[kDecayMetaSBase + gen];
    const int64_t tot = off_all[ib + gen + n];
    const int64_t st = tot >> 32, ut = tot & 0xFFFFFFFFll;
    int64_t next_n = ut;
    const int64_t next_sb = sb + st, next_ib = ib + n;
    if (meta[kDecayMetaFlags] == 0 && next_sb > s_cap) {
        meta[kDecayMetaFlags] |= 1;
        meta[kDecayMetaNeedS] = next_sb;
    }
    if (meta[kDecayMetaFlags] == 0 && ut > u_cap) {
        meta[kDecayMetaFlags] |= 2;
        meta[kDecayMetaNeedU] = ut;
    }
    if (meta[kDecayMetaFlags] == 0 && next_ib + ut > i_cap) {
        meta[kDecayMetaFlags] |= 8;
        meta[kDecayMetaNeedI] = next_ib + ut;
    }
    if (meta[kDecayMetaFlags] == 0 && gen + 1 >= g_max && ut > 0) meta[kDecayMetaFlags] |= 4;
    if (meta[kDecayMetaFlags] != 0) next_n = 0;
    meta[kDecayMetaNIn + gen + 1] = next_n;
    meta[kDecayMetaSBase + gen + 1] = next_sb;
    meta[kDecayMetaIBase + gen + 1] = next_ib;
    if (ut > meta[kDecayMetaMaxU]) meta[kDecayMetaMaxU] = ut;
}

// Per event: its stable products in this generation (scnt) and its input
// range in the next one (the unstable products of its inputs, contiguous
// because the inputs are grouped by event).
__global__ void dk_next_bounds_kernel(const int64_t* __restrict__ meta, uint32_t gen,
                                      const int64_t* __restrict__ off_all, int n_events, uint32_t g_max,
                                      int64_t* __restrict__ first, int64_t* __restrict__ last,
                                      int64_t* __restrict__ scnt) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_events || meta[kDecayMetaFlags] != 0) return;
    const int64_t r = static_cast<int64_t>(gen) * n_events + e;
    const int64_t f = first[r];
    int64_t sc = 0;
    if (f >= 0) {
        const int64_t* off = off_all + meta_ib(meta, gen) + gen;
        const int64_t a = off[f], b = off[last[r]];
        sc = (b >> 32) - (a >> 32);
        const int64_t ua = a & 0xFFFFFFFFll, ub = b & 0xFFFFFFFFll;
        if (ub > ua && gen + 1 < g_max) {
            first[r + n_events] = ua;
            last[r + n_events] = ub;
        }
    }
    scnt[r] = sc;
}

// ---- the final lists ----------------------------------------------------

// per event: its stable products over generations g < n_gen
__global__ void dk_event_totals_kernel(const int64_t* __restrict__ scnt, int n_gen, int n_events,
                                       int32_t* __restrict__ tot) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_events) return;
    int64_t k = 0;
    for (int g = 0; g < n_gen; g++) k += scnt[static_cast<int64_t>(g) * n_events + e];
    tot[e] = static_cast<int32_t>(k);
}

// shift[g][e] = final place of event e's first stable product of generation
// g, less the stable scan offset of the event's first input in g
__global__ void dk_shift_kernel(const int64_t* __restrict__ scnt, const int64_t* __restrict__ first,
                                const int64_t* __restrict__ off_all, const int64_t* __restrict__ meta,
                                const int64_t* __restrict__ evoff, int n_gen, int n_events,
                                int64_t* __restrict__ shift) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_events) return;
    int64_t b = evoff[e];
    for (int g = 0; g < n_gen; g++) {
        const int64_t r = static_cast<int64_t>(g) * n_events + e;
        const int64_t f = first[r];
        if (f >= 0) shift[r] = b - (off_all[meta_ib(meta, static_cast<uint32_t>(g)) + g + f] >> 32);
        b += scnt[r];
    }
}

}  // namespace

cudaError_t launch_decay_first_generation(const int64_t* evoff, int n_events, const DecayBuffers& b,
                                          cudaStream_t s) {
    if (n_events <= 0) return cudaSuccess;
    event_ids_kernel<<<n_events, 128, 0, s>>>(evoff, n_events, b.ev);
    dk_first_gen_kernel<<<(n_events + 255) / 256, 256, 0, s>>>(evoff, n_events, b.first, b.last);
    return cudaGetLastError();
}

cudaError_t launch_decay_count_generation(const DevConfig& cfg, const DecayTablesDev& t, uint32_t gen,
                                          const DecayBuffers& b, int n_events, int num_sms,
                                          cudaStream_t s) {
    // grid-stride kernels launched with what fits on the SMs at once (eight
    // blocks of 256)
    const int grid = num_sms * 8;
    const int64_t* first = b.first + static_cast<int64_t>(gen) * n_events;
    decay_count_kernel<<<grid, kDecayThreads, 0, s>>>(cfg, t, gen, b.rec0, b.pid, b.ev, first, b.meta,
                                                      b.chan, b.cnt);
    dk_tile_sum_kernel<<<grid, kDkScanThreads, 0, s>>>(b.cnt, b.meta, gen, b.tiles);
    dk_tile_offset_kernel<<<1, kDkScanThreads, 0, s>>>(b.tiles, b.meta, gen, b.off);
    dk_tile_scan_kernel<<<grid, kDkScanThreads, 0, s>>>(t, b.cnt, b.meta, gen, b.tiles, b.chan, b.ev, b.pid,
                                                        b.i_cap, b.off);
    dk_advance_kernel<<<1, 32, 0, s>>>(b.meta, gen, b.off, b.s_cap, b.u_cap, b.i_cap, b.g_max);
    dk_next_bounds_kernel<<<(n_events + 255) / 256, 256, 0, s>>>(b.meta, gen, b.off, n_events, b.g_max,
                                                                 b.first, b.last, b.scnt);
    return cudaGetLastError();
}

cudaError_t launch_decay_layout(const DecayBuffers& b, int n_gen, int n_events, int32_t* ev_tot,
                                int64_t* tiles, int64_t* evoff, cudaStream_t s) {
    if (n_events <= 0) return cudaSuccess;
    const unsigned eb = static_cast<unsigned>((n_events + 255) / 256);
    dk_event_totals_kernel<<<eb, 256, 0, s>>>(b.scnt, n_gen, n_events, ev_tot);
    cudaError_t e = launch_offsets_scan(ev_tot, n_events, tiles, evoff, s);
    if (e != cudaSuccess) return e;
    dk_shift_kernel<<<eb, 256, 0, s>>>(b.scnt, b.first, b.off, b.meta, evoff, n_gen, n_events, b.shift);
    return cudaGetLastError();
}

cudaError_t launch_decay_write_generation(const DevConfig& cfg, const DecayTablesDev& t, uint32_t gen,
                                          int64_t n, int64_t ib, const HadronRec* in, HadronRec* out_u,
                                          const DecayBuffers& b, int n_events, int num_sms,
                                          HadronRec* out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    // three blocks of 256 fit per SM at 80 registers; small generations get
    // one warp per 32 inputs at most
    const int64_t want = (n + kDecayThreads - 1) / kDecayThreads;
    const int grid = static_cast<int>(std::min<int64_t>(want, static_cast<int64_t>(num_sms) * 3));
    const int64_t r = static_cast<int64_t>(gen) * n_events;
    decay_write_kernel<<<grid, kDecayThreads, 0, s>>>(cfg, t, gen, n, in, b.ev + ib, b.first + r,
                                                      b.chan + ib, b.off + ib + gen, b.shift + r, out,
                                                      out_u, b.failures);
    return cudaGetLastError();
}

}  // namespace iss
