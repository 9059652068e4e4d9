/* Test infrastructure only -- oracle part 2c: FP64 replay of the GPU's
 * resonance decays on the same Philox streams.  The reference's algorithm it
 * restates:
 *   FSSW::perform_resonance_feed_down,   src/FSSW.cpp:1746-1779 (per event, a
 *       FIFO list: the sampled hadrons, then every unstable daughter appended
 *       in order; stable products go to the output in that order)
 *   particle_decay::perform_decays,      src/particle_decay.cpp:266-330
 *       (a stable or unknown hadron passes unchanged; a channel by cumulated
 *       branching ratios against one uniform; 2- and 3-body channels only)
 *   particle_decay::perform_two_body_decay,   src/particle_decay.cpp:353-419
 *   particle_decay::perform_three_body_decay, src/particle_decay.cpp:423-513
 *       (pole mass, rejection on (E1, E2), three angles, lifetime gamma/Gamma
 *       in fm, boost with the mother's velocity)
 *
 * The FIFO list is processed breadth first: generation g is the set of list
 * entries appended while generation g-1 was processed, so the output order
 * is the same when generations are walked one after the other.  The random
 * numbers follow the GPU's keys: Philox4x32-10 with counter (draw, index of
 * the hadron in its event's generation list, event, generation | 4 << 16):
 *   draw 0       the channel: m = (x >> 5) 2^26 + (y >> 6), the first channel
 *                with m < ceil(2^53 x the partial sum of branching ratios);
 *   draw 1       the angles and the lifetime: azimuths 2 pi (u - 1/2) from x
 *                (and y for the third angle of 3-body decays), cos theta from
 *                y (2-body) or z (3-body), the lifetime from w;
 *   draws 16+it  3-body (E1, E2) candidates, (x, y) then (z, w).
 * Kinematics are computed in FP64 from the float records, as the reference
 * does in double; the GPU computes in FP32, so momenta agree to rounding and
 * a 3-body candidate at the edge of the (E1, E2) region can be accepted by
 * one and not the other (counted by the test). */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"
#include "philox.h"

#define ORC_TAG_DECAY 4u
#define ORC_TWO_PI 6.28318530717958647692

static void dblock(const uint32_t key[2], uint32_t draw, uint32_t i, uint32_t e, uint32_t gen,
                   uint32_t w[4]) {
    const uint32_t ctr[4] = {draw, i, e, gen | (ORC_TAG_DECAY << 16)};
    orc_philox4x32_10(ctr, key, w);
}

/* the first particle with this pid (particle_decay's lookups), -1 if none */
static int find_pid(const orc_dparticle* parts, int32_t n_parts, int32_t pid) {
    for (int32_t i = 0; i < n_parts; i++)
        if (parts[i].pid == pid) return i;
    return -1;
}

static int daughter_stable(const orc_dparticle* parts, int32_t idx) {
    return idx < 0 || parts[idx].stable;
}

typedef struct {
    int32_t pid;
    double mass, E, px, py, pz, t, x, y, z;
} rec;

static rec to_rec(const orc_hadron* h) {
    rec r;
    r.pid = h->pid;
    r.mass = h->mass;
    r.E = h->E; r.px = h->px; r.py = h->py; r.pz = h->pz;
    r.t = h->t; r.x = h->x; r.y = h->y; r.z = h->z;
    return r;
}

static orc_hadron to_hadron(const rec* r) {
    orc_hadron h;
    h.pid = r->pid;
    h.mass = (float)r->mass;
    h.E = (float)r->E; h.px = (float)r->px; h.py = (float)r->py; h.pz = (float)r->pz;
    h.t = (float)r->t; h.x = (float)r->x; h.y = (float)r->y; h.z = (float)r->z;
    return h;
}

/* boost of a rest-frame (E, p) with the mother's velocity: the reference's
 * E' = gamma (E + v.p), p' = p + ((gamma - 1) v.p / v^2 + gamma E) v with
 * v = p_m/E_m, gamma = 1/sqrt(1 - v^2) (src/particle_decay.cpp:390-400),
 * written with the mother's four-velocity u = p_m/m, gamma = E_m/m:
 * E' = gamma E + u.p, p' = p + (E + u.p/(gamma + 1)) u.  For an on-shell
 * mother the two are the same boost; from float records the second keeps
 * its digits where 1 - v^2 cancels (gamma ~ 80 loses about 4e-4 of gamma in
 * the first form), and it is the GPU's form. */
static void boost(const rec* m, double E, double px, double py, double pz, rec* d) {
    const double inv = 1.0 / m->mass;
    const double ux = m->px * inv, uy = m->py * inv, uz = m->pz * inv, gamma = m->E * inv;
    const double up = ux * px + uy * py + uz * pz;
    const double c = E + up / (gamma + 1.0);
    d->E = gamma * E + up;
    d->px = px + c * ux;
    d->py = py + c * uy;
    d->pz = pz + c * uz;
}

/* the products of mother m (index ie in its event's generation list) through
 * channel ch of particle type; returns their number (0, 2 or 3) */
static int decay_one(const orc_dparticle* parts, const orc_dchannel* ch, int type, const rec* m,
                     const uint32_t key[2], uint32_t ie, uint32_t eg, uint32_t gen, rec* out,
                     int64_t* failures) {
    const int n = ch->n_daughters;
    const double M = parts[type].mass;
    const double width = parts[type].width;
    double md[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < n; k++) md[k] = ch->daughter[k] >= 0 ? parts[ch->daughter[k]].mass : 0.0;
    uint32_t w1[4];
    dblock(key, 1u, ie, eg, gen, w1);
    double E[3], px[3], py[3], pz[3];
    if (n == 2) {
        const double m1 = md[0], m2 = md[1];
        const double a = M * M - m1 * m1 - m2 * m2;
        double disc = a * a - 4.0 * m1 * m1 * m2 * m2;
        if (disc < 0.0) disc = 0.0;
        const double p = sqrt(disc) / (2.0 * M);
        const double phi = ORC_TWO_PI * (orc_u01(w1[0]) - 0.5);
        const double cth = 2.0 * (orc_u01(w1[1]) - 0.5);
        const double sth = sqrt(fmax(1.0 - cth * cth, 0.0));
        px[0] = p * sth * cos(phi);
        py[0] = p * sth * sin(phi);
        pz[0] = p * cth;
        E[0] = sqrt(p * p + m1 * m1);
        px[1] = -px[0];
        py[1] = -py[0];
        pz[1] = -pz[0];
        E[1] = sqrt(p * p + m2 * m2);
    } else {
        const double m1 = md[0], m2 = md[1], m3 = md[2];
        const double span = M - m1 - m2 - m3;
        double E1 = m1, E2 = m2, p1 = 0.0, p2 = 0.0, c12 = 0.0;
        int ok = 0;
        for (int it = 0; it < 50000 && !ok; it++) {
            uint32_t w[4];
            dblock(key, 16u + (uint32_t)it, ie, eg, gen, w);
            for (int h = 0; h < 2 && !ok; h++) {
                E1 = orc_u01(h ? w[2] : w[0]) * span + m1;
                E2 = orc_u01(h ? w[3] : w[1]) * span + m2;
                if (E1 + E2 > M) continue;
                p1 = sqrt(fmax(E1 * E1 - m1 * m1, 0.0));
                p2 = sqrt(fmax(E2 * E2 - m2 * m2, 0.0));
                const double E3 = M - E1 - E2;
                c12 = (E3 * E3 - p1 * p1 - p2 * p2 - m3 * m3) / (2.0 * p1 * p2);
                ok = (c12 >= -1.0 && c12 <= 1.0);
            }
        }
        if (!ok) {
            (*failures)++;
            c12 = 1.0;
        }
        const double tp2x = p2 * sqrt(fmax(1.0 - c12 * c12, 0.0)), tp2z = p2 * c12;
        const double tp3x = -tp2x, tp3z = -(p1 + tp2z);
        const double phi = ORC_TWO_PI * (orc_u01(w1[0]) - 0.5);
        const double ksi = ORC_TWO_PI * (orc_u01(w1[1]) - 0.5);
        const double cth = 2.0 * orc_u01(w1[2]) - 1.0;
        const double sphi = sin(phi), cphi = cos(phi), sksi = sin(ksi), cksi = cos(ksi);
        const double sth = sqrt(fmax(1.0 - cth * cth, 0.0));
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
            E[k] = sqrt(md[k] * md[k] + px[k] * px[k] + py[k] * py[k] + pz[k] * pz[k]);
    }
    double life = 1e10;
    if (width > 1e-10) {
        const double tau0 = m->E / M / width;
        life = -tau0 * log(orc_u01_pos(w1[3])) * 0.19733;
    }
    for (int k = 0; k < n; k++) {
        rec* d = out + k;
        const int di = ch->daughter[k];
        d->pid = di >= 0 ? parts[di].pid : 0;
        d->mass = md[k];
        boost(m, E[k], px[k], py[k], pz[k], d);
        d->t = m->t + life;
        d->x = m->x + m->px / m->E * life;
        d->y = m->y + m->py / m->E * life;
        d->z = m->z + m->pz / m->E * life;
    }
    return n;
}

int64_t orc_decay_replay(const orc_dparticle* parts, int32_t n_parts, const orc_dchannel* chans,
                         uint64_t seed, int64_t event_offset, int32_t n_events, const int64_t* ev_off,
                         const orc_hadron* in, int64_t capacity, orc_hadron* out, int64_t* out_off,
                         int64_t* failures) {
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    int64_t w = 0;
    *failures = 0;
    /* the current generation (read) and the next one (appended) */
    rec* cur = NULL;
    rec* next = NULL;
    int64_t cap_cur = 0, cap_next = 0;
    int64_t status = 0;
    for (int32_t e = 0; e < n_events && status == 0; e++) {
        out_off[e] = w;
        const uint32_t eg = (uint32_t)(event_offset + e);
        int64_t n = ev_off[e + 1] - ev_off[e];
        if (n > cap_cur) {
            free(cur);
            cap_cur = n;
            cur = (rec*)malloc(sizeof(rec) * (size_t)cap_cur);
            if (!cur) {
                status = -2;
                break;
            }
        }
        for (int64_t i = 0; i < n; i++) cur[i] = to_rec(in + ev_off[e] + i);
        for (uint32_t gen = 0; n > 0 && status == 0; gen++) {
            int64_t nn = 0;
            for (int64_t i = 0; i < n && status == 0; i++) {
                const rec* m = cur + i;
                const int type = find_pid(parts, n_parts, m->pid);
                if (type < 0 || parts[type].stable) {
                    if (w >= capacity) {
                        status = -1;
                        break;
                    }
                    out[w++] = to_hadron(m);
                    continue;
                }
                uint32_t w0[4];
                dblock(key, 0u, (uint32_t)i, eg, gen, w0);
                const uint64_t mm = ((uint64_t)(w0[0] >> 5) << 26) | (uint64_t)(w0[1] >> 6);
                int c = -1;
                for (int k = 0; k < parts[type].n_channels; k++) {
                    if (mm < chans[parts[type].first_channel + k].cum53) {
                        c = parts[type].first_channel + k;
                        break;
                    }
                }
                /* no channel reached the uniform, or not a 2- or 3-body
                 * channel: no product */
                if (c < 0 || (chans[c].n_daughters != 2 && chans[c].n_daughters != 3)) continue;
                rec prod[3];
                const int np = decay_one(parts, chans + c, type, m, key, (uint32_t)i, eg, gen, prod, failures);
                for (int k = 0; k < np; k++) {
                    if (daughter_stable(parts, chans[c].daughter[k])) {
                        if (w >= capacity) {
                            status = -1;
                            break;
                        }
                        out[w++] = to_hadron(prod + k);
                    } else {
                        if (nn >= cap_next) {
                            const int64_t cap = 2 * cap_next + 64;
                            rec* b = (rec*)realloc(next, sizeof(rec) * (size_t)cap);
                            if (!b) {
                                status = -2;
                                break;
                            }
                            next = b;
                            cap_next = cap;
                        }
                        next[nn++] = prod[k];
                    }
                }
            }
            /* the next generation becomes the current one */
            rec* t = cur;
            cur = next;
            next = t;
            const int64_t tc = cap_cur;
            cap_cur = cap_next;
            cap_next = tc;
            n = nn;
        }
    }
    if (status == 0) out_off[n_events] = w;
    free(cur);
    free(next);
    return status != 0 ? status : w;
}
