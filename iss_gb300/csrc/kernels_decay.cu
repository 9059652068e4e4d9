// Resonance decays of the sampled hadrons (FSSW::perform_resonance_feed_down,
// src/FSSW.cpp:1746-1779, with particle_decay::perform_decays and the two-
// and three-body kinematics of src/particle_decay.cpp:265-513).
//
// The reference walks each event's list: a stable hadron goes to the output,
// an unstable one decays and its daughters go to the output (stable) or to
// the end of the list (unstable).  The output of an event is therefore, in
// order, the stable products of the sampled hadrons, then those of their
// unstable daughters, then of the granddaughters, and so on.  Here each such
// generation is one pass over all events at once: a count kernel (channel
// choice, stable and unstable products per hadron), two exclusive scans, and
// a write kernel that puts stable products into this generation's output and
// unstable ones into the next generation's input, both in order.  The final
// list of each event is the concatenation of its generations' outputs.
//
// Every random number comes from Philox4x32-10 with counter
// (draw, index of the hadron in its event's generation list, event,
// generation | kTagDecay << 16): results do not depend on thread mapping.
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "kernels.h"

namespace iss {

namespace {

constexpr int kDecayThreads = 256;
constexpr uint32_t kTagDecay = 4u;
constexpr int kThreeBodyTries = 100000;

__device__ __forceinline__ uint4 dblock(uint32_t draw, uint32_t i, uint32_t e, uint32_t gen,
                                        uint32_t k0, uint32_t k1) {
    return philox4x32_10(make_uint4(draw, i, e, gen | (kTagDecay << 16)), k0, k1);
}

// index of pid in the decay table (pids sorted with their indices), -1 if absent
__device__ __forceinline__ int lookup(const DecayTablesDev& t, int pid) {
    int lo = 0, hi = t.n_particles - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int v = t.sorted_pid[mid];
        if (v == pid) return t.sorted_idx[mid];
        if (v < pid) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

// The channel of an unstable particle (cumulated branching ratios against one
// uniform, src/particle_decay.cpp:283-293), or -1 when the ratios do not
// reach the uniform.
__device__ __forceinline__ int pick_channel(const DecayTablesDev& t, int type, double u) {
    const int c0 = t.particles[type].first_channel, nc = t.particles[type].n_channels;
    double cum = 0.0;
    for (int c = 0; c < nc; c++) {
        cum += t.channels[c0 + c].branching_ratio;
        if (cum > u) return c0 + c;
    }
    return -1;
}

struct DecayPlan {
    int type, channel, n;      // n: daughters (0: none written, 1: the particle itself)
};

__device__ DecayPlan plan(const DecayTablesDev& t, const DevConfig& cfg, int pid, uint32_t i,
                          uint32_t eg, uint32_t gen) {
    DecayPlan d{};
    d.type = lookup(t, pid);
    d.channel = -1;
    if (d.type < 0 || t.particles[d.type].stable) {
        d.n = 1;
        return d;
    }
    const uint4 w = dblock(0u, i, eg, gen, cfg.key0, cfg.key1);
    d.channel = pick_channel(t, d.type, u53(w.x, w.y));
    const int nd = d.channel >= 0 ? t.channels[d.channel].n_daughters : 0;
    // the reference decays into two or three bodies only; other channels
    // leave no product (src/particle_decay.cpp:294-330)
    d.n = (nd == 2 || nd == 3) ? nd : 0;
    return d;
}

__device__ __forceinline__ bool daughter_stable(const DecayTablesDev& t, int idx) {
    return idx < 0 || t.particles[idx].stable;
}

__global__ void __launch_bounds__(kDecayThreads)
decay_count_kernel(DevConfig cfg, DecayTablesDev t, uint32_t gen, const HadronRec* __restrict__ in,
                   const int32_t* __restrict__ ev, const int64_t* __restrict__ first, int64_t n,
                   int32_t* __restrict__ n_stable, int32_t* __restrict__ n_unstable) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int e = ev[i];
    const DecayPlan d = plan(t, cfg, in[i].pid, static_cast<uint32_t>(i - first[e]),
                             cfg.event_offset + static_cast<uint32_t>(e), gen);
    int s = 0, u = 0;
    if (d.channel < 0) {
        s = d.n;   // stable (or no channel: nothing)
    } else {
        for (int k = 0; k < d.n; k++) {
            if (daughter_stable(t, t.channels[d.channel].daughter[k])) s++; else u++;
        }
    }
    n_stable[i] = s;
    n_unstable[i] = u;
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

__global__ void __launch_bounds__(kDecayThreads)
decay_write_kernel(DevConfig cfg, DecayTablesDev t, uint32_t gen, const HadronRec* __restrict__ in,
                   const int32_t* __restrict__ ev, const int64_t* __restrict__ first, int64_t n,
                   const int64_t* __restrict__ s_off, const int64_t* __restrict__ u_off,
                   HadronRec* __restrict__ out_s, int32_t* __restrict__ ev_s,
                   HadronRec* __restrict__ out_u, int32_t* __restrict__ ev_u,
                   unsigned long long* __restrict__ failures) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int e = ev[i];
    const uint32_t ie = static_cast<uint32_t>(i - first[e]);
    const uint32_t eg = cfg.event_offset + static_cast<uint32_t>(e);
    const HadronRec m = in[i];
    const DecayPlan d = plan(t, cfg, m.pid, ie, eg, gen);
    int64_t ps = s_off[i], pu = u_off[i];
    if (d.channel < 0) {
        if (d.n == 1) {
            out_s[ps] = m;
            ev_s[ps] = e;
        }
        return;
    }
    if (d.n == 0) return;
    const DecayChannel& ch = t.channels[d.channel];
    const DecayParticle& mp = t.particles[d.type];
    const float M = mp.mass;       // pole mass (the reference does not sample Breit-Wigner)
    float md[3];
    for (int k = 0; k < d.n; k++) {
        const int di = ch.daughter[k];
        md[k] = di >= 0 ? t.particles[di].mass : 0.0f;
    }
    float E[3], px[3], py[3], pz[3];
    float life;
    const uint4 w1 = dblock(1u, ie, eg, gen, cfg.key0, cfg.key1);
    if (d.n == 2) {
        const float m1 = md[0], m2 = md[1];
        const float a = M * M - m1 * m1 - m2 * m2;
        const float p = sqrtf(fmaxf(a * a - 4.0f * m1 * m1 * m2 * m2, 0.0f)) / (2.0f * M);
        float sphi, cphi;
        sincospif(2.0f * u01f(w1.x), &sphi, &cphi);
        const float cth = 2.0f * (u01f(w1.y) - 0.5f);
        const float sth = sqrtf(fmaxf(1.0f - cth * cth, 0.0f));
        px[0] = p * sth * cphi;
        py[0] = p * sth * sphi;
        pz[0] = p * cth;
        E[0] = sqrtf(p * p + m1 * m1);
        px[1] = -px[0];
        py[1] = -py[0];
        pz[1] = -pz[0];
        E[1] = sqrtf(p * p + m2 * m2);
    } else {
        // phase space by rejection on (E1, E2) (src/particle_decay.cpp:445-458)
        const float m1 = md[0], m2 = md[1], m3 = md[2];
        const float span = M - m1 - m2 - m3;
        float E1 = m1, E2 = m2, p1 = 0.f, p2 = 0.f, c12 = 0.f;
        bool ok = false;
        for (int it = 0; it < kThreeBodyTries && !ok; it++) {
            const uint4 w = dblock(16u + static_cast<uint32_t>(it), ie, eg, gen, cfg.key0, cfg.key1);
            E1 = u01f(w.x) * span + m1;
            E2 = u01f(w.y) * span + m2;
            if (E1 + E2 > M) continue;
            p1 = sqrtf(fmaxf(E1 * E1 - m1 * m1, 0.0f));
            p2 = sqrtf(fmaxf(E2 * E2 - m2 * m2, 0.0f));
            const float E3 = M - E1 - E2;
            c12 = (E3 * E3 - p1 * p1 - p2 * p2 - m3 * m3) / (2.0f * p1 * p2);
            ok = (c12 >= -1.0f && c12 <= 1.0f);
        }
        if (!ok) {
            atomicAdd(failures, 1ull);
            c12 = 1.0f;
        }
        const float tp2x = p2 * sqrtf(fmaxf(1.0f - c12 * c12, 0.0f)), tp2z = p2 * c12;
        const float tp3x = -tp2x, tp3z = -(p1 + tp2z);
        float sphi, cphi, sksi, cksi;
        sincospif(2.0f * u01f(w1.x), &sphi, &cphi);
        sincospif(2.0f * u01f(w1.y), &sksi, &cksi);
        const float cth = 2.0f * u01f(w1.z) - 1.0f;
        const float sth = sqrtf(fmaxf(1.0f - cth * cth, 0.0f));
        px[0] = -p1 * sth * cksi;
        py[0] = p1 * sth * sksi;
        pz[0] = p1 * cth;
        px[1] = tp2x * (cphi * cth * cksi - sphi * sksi) - tp2z * sth * cksi;
        py[1] = tp2x * (-cphi * cth * sksi - sphi * cksi) + tp2z * sth * sksi;
        pz[1] = tp2x * (cphi * sth) + tp2z * cth;
        px[2] = tp3x * (cphi * cth * cksi - sphi * sksi) - tp3z * sth * cksi;
        py[2] = tp3x * (-cphi * cth * sksi - sphi * cksi) + tp3z * sth * sksi;
        pz[2] = tp3x * cphi * sth + tp3z * cth;
        for (int k = 0; k < 3; k++)
            E[k] = sqrtf(md[k] * md[k] + px[k] * px[k] + py[k] * py[k] + pz[k] * pz[k]);
    }
    // life time gamma / Gamma in fm (src/particle_decay.cpp:396-401)
    life = 1e10f;
    if (mp.width > 1e-10f) {
        const float tau0 = m.E / M / mp.width;
        life = -tau0 * __logf(u01f_pos(w1.w)) * 0.19733f;
    }
    const float inv = 1.0f / m.E;
    const float dt = m.t + life, dx = m.x + m.px * inv * life, dy = m.y + m.py * inv * life,
                dz = m.z + m.pz * inv * life;
    const Lorentz L = velocity(m);
    for (int k = 0; k < d.n; k++) {
        HadronRec r;
        const int di = ch.daughter[k];
        r.pid = di >= 0 ? t.particles[di].pid : 0;
        r.mass = md[k];
        boost(L, E[k], px[k], py[k], pz[k], &r.E, &r.px, &r.py, &r.pz);
        r.t = dt;
        r.x = dx;
        r.y = dy;
        r.z = dz;
        if (daughter_stable(t, di)) {
            out_s[ps] = r;
            ev_s[ps] = e;
            ps++;
        } else {
            out_u[pu] = r;
            ev_u[pu] = e;
            pu++;
        }
    }
}

// first[e] = index of event e's first element in an event-sorted array, and
// last[e] = one past its last (both stay -1 for absent events)
__global__ void event_bounds_kernel(const int32_t* __restrict__ ev, int64_t n,
                                    int64_t* __restrict__ first, int64_t* __restrict__ last) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int e = ev[i];
    if (i == 0 || ev[i - 1] != e) first[e] = i;
    if (i == n - 1 || ev[i + 1] != e) last[e] = i + 1;
}

// event ids of the sampled records from the event offsets
__global__ void event_ids_kernel(const int64_t* __restrict__ off, int n_events,
                                 int32_t* __restrict__ ev) {
    const int e = blockIdx.x;
    if (e >= n_events) return;
    for (int64_t i = off[e] + threadIdx.x; i < off[e + 1]; i += blockDim.x) ev[i] = e;
}

// out[base[e] + i - first[e]] = in[i]
__global__ void gather_kernel(const HadronRec* __restrict__ in, const int32_t* __restrict__ ev,
                              const int64_t* __restrict__ first, const int64_t* __restrict__ base,
                              int64_t n, HadronRec* __restrict__ out) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int e = ev[i];
    out[base[e] + (i - first[e])] = in[i];
}

unsigned grid_for(int64_t n) { return static_cast<unsigned>((n + kDecayThreads - 1) / kDecayThreads); }

}  // namespace

cudaError_t launch_event_ids(const int64_t* off, int n_events, int32_t* ev, cudaStream_t s) {
    if (n_events <= 0) return cudaSuccess;
    event_ids_kernel<<<n_events, 128, 0, s>>>(off, n_events, ev);
    return cudaGetLastError();
}

cudaError_t launch_event_bounds(const int32_t* ev, int64_t n, int n_events, int64_t* first,
                                int64_t* last, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(first, 0xFF, sizeof(int64_t) * n_events, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(last, 0xFF, sizeof(int64_t) * n_events, s);
    if (e != cudaSuccess || n <= 0) return e;
    event_bounds_kernel<<<grid_for(n), kDecayThreads, 0, s>>>(ev, n, first, last);
    return cudaGetLastError();
}

cudaError_t launch_decay_count(const DevConfig& cfg, const DecayTablesDev& t, uint32_t gen,
                               const HadronRec* in, const int32_t* ev, const int64_t* first,
                               int64_t n, int32_t* n_stable, int32_t* n_unstable, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    decay_count_kernel<<<grid_for(n), kDecayThreads, 0, s>>>(cfg, t, gen, in, ev, first, n, n_stable,
                                                              n_unstable);
    return cudaGetLastError();
}

cudaError_t launch_decay_write(const DevConfig& cfg, const DecayTablesDev& t, uint32_t gen,
                               const HadronRec* in, const int32_t* ev, const int64_t* first,
                               int64_t n, const int64_t* s_off, const int64_t* u_off,
                               HadronRec* out_s, int32_t* ev_s, HadronRec* out_u, int32_t* ev_u,
                               unsigned long long* failures, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    decay_write_kernel<<<grid_for(n), kDecayThreads, 0, s>>>(cfg, t, gen, in, ev, first, n, s_off,
                                                              u_off, out_s, ev_s, out_u, ev_u,
                                                              failures);
    return cudaGetLastError();
}

cudaError_t launch_gather(const HadronRec* in, const int32_t* ev, const int64_t* first,
                          const int64_t* base, int64_t n, HadronRec* out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    gather_kernel<<<grid_for(n), kDecayThreads, 0, s>>>(in, ev, first, base, n, out);
    return cudaGetLastError();
}

}  // namespace iss
