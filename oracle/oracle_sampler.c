/* Test infrastructure only -- oracle part 2b: FP64 replay of the GPU momentum
 * sampler on the same Philox streams.  The reference's algorithm it restates:
 *   FSSW::sample_using_dN_dxtdy_4all_particles_conventional, src/FSSW.cpp:970-1049
 *   FSSW::sample_momemtum_from_a_fluid_cell,                 src/FSSW.cpp:1852-1966
 *   FSSW::get_deltaf_bulk,                                   src/FSSW.cpp:1795-1849
 *   MomentumSamplerShell / MomentumSamplerBase / Boson-, FermionMomentumSampler
 *       (|p| ~ p^2 f(E) with the table ranges of src/BosonMomentumSampler.cpp:15-17,
 *        src/FermionMomentumSampler.cpp:15-17 and src/MomentumSamplerShell.cpp:24-48)
 *   FSSW::boost_vector_back_to_lab_frame, src/FSSW.cpp:2001-2010
 *   FSSW::add_one_sampled_particle,       src/FSSW.cpp:1969-1996
 *
 * The GPU proposes |p| from an exact Gamma mixture matching (E^2 - m^2/2)
 * exp(-(E - mu)/T) (for bosons without diffusion or the compat-fermion
 * factor (E^2 - m^2/2) times the first three terms of the Bose-Einstein
 * series, exp(-n (E - mu)/T) for n = 1, 2, 3, term n being the same mixture
 * at rate n), the direction from the Cooper-Frye flux factor itself
 * (linear in the cosine of the angle to the spatial part of dsigma in the rest
 * frame, inverse CDF), and folds the quantum-statistics, pE/(E^2 - m^2/2),
 * |p|-dependent flux remainder and delta-f acceptances into one uniform per
 * try; the resulting density is the reference's p^2 f(E) x accept.  This file restates that
 * algorithm draw for draw so that the GPU output can be compared hadron by
 * hadron. */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"
#include "philox.h"

#define ORC_PI 3.14159265358979323846

typedef struct {
    /* cell */
    double tau, xpt, ypt, eta;
    double da[4], u[4];
    double E, T, P, nB, muB, muS, muQ, Pi;
    double pxx, pxy, pxz, pyy, pyz, qx, qy, qz;
    double vis0, vis1, vis2, kappa;
} orc_cell;

static void orc_load_cell(const float* lrf28, const float* coef4, int64_t l, orc_cell* c) {
    const float* s = lrf28 + 28 * l;
    c->tau = s[0]; c->xpt = s[1]; c->ypt = s[2]; c->eta = s[3];
    for (int k = 0; k < 4; k++) { c->da[k] = s[4 + k]; c->u[k] = s[8 + k]; }
    c->E = s[12]; c->T = s[13]; c->P = s[14]; c->nB = s[15];
    c->muB = s[16]; c->muS = s[17]; c->muQ = s[18]; c->Pi = s[19];
    c->pxx = s[20]; c->pxy = s[21]; c->pxz = s[22]; c->pyy = s[23]; c->pyz = s[24];
    c->qx = s[25]; c->qy = s[26]; c->qz = s[27];
    c->vis0 = coef4[4 * l + 0]; c->vis1 = coef4[4 * l + 1];
    c->vis2 = coef4[4 * l + 2]; c->kappa = coef4[4 * l + 3];
}

/* Cell draw of the GPU sampler on the fixed-point CDF C[0..n] (orc_cdf):
 * v = floor(r * Q / 2^64) for 64 random bits r, and the cell is the largest i
 * with C[i] <= v, i.e. C[i] <= v < C[i+1] -- binarySearch
 * (src/arsenal.cpp:644-678) on integer sums. */
static int64_t orc_search(const uint64_t* cdf, int64_t n, uint64_t Q, uint64_t r) {
    const uint64_t v = (uint64_t)(((unsigned __int128)r * Q) >> 64);
    int64_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) / 2;
        if (cdf[mid] <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

typedef struct {
    double m, mt, mu, mut, a, T, beta;
    int boson;
    double Kmax, w3, w2, W;
    double W1, W12, r2;    /* bosons: weights of the exp(-E~) term and of the
                              first two terms, 4 exp(a) */
    double qa;             /* 1 - exp(-a), 1 - exp(-3a) with bose3 */
    int bose3;             /* the three-term Bose proposal */
    int compat;            /* reproduce the reference's truncated/buggy series */
    double rmax;
    double c_poly;         /* mu~^2 - m~^2/2 */
    int status;            /* 0 ok, 1 m/T - mu/T off the momentum tables */
} orc_prop;

/* Sampler selection and table ranges, src/MomentumSamplerShell.cpp:24-48,
 * src/BosonMomentumSampler.cpp:15-17, src/FermionMomentumSampler.cpp:15-17,
 * range check src/MomentumSamplerBase.cpp:32-43. */
static void orc_setup(const orc_cfg* cfg, double m, int sign, double mu_raw, double T,
                      orc_prop* p) {
    p->m = m;
    p->T = T;
    p->beta = 1.0 / T;
    p->mu = mu_raw < m ? mu_raw : m;
    p->mt = m * p->beta;
    p->mut = p->mu * p->beta;
    p->a = (m - p->mu) * p->beta;
    p->boson = (sign == -1);
    const int sampler = p->a < 30.0 ? 0 : (p->a < 50.0 ? 1 : 2);
    double e0, de;
    int npts;
    if (p->boson) {
        e0 = (sampler == 0 ? 0.05 : (sampler == 1 ? 30.0 : 50.0)) + 0.05;
        de = 0.05;
        npts = 1001;
    } else {
        e0 = (sampler == 0 ? 0.0 : (sampler == 1 ? 30.0 : 50.0));
        de = 0.02;
        npts = 2001;
    }
    const double emax = e0 + (npts - 1) * de;
    const int idx_min = (int)((p->a - e0) / de);
    p->status = (idx_min < 0 || idx_min >= npts - 1) ? 1 : 0;
    p->Kmax = emax - p->a;
    p->w3 = 2.0;
    p->w2 = 2.0 * p->mt;
    p->W = p->w3 + p->w2 + 0.5 * p->mt * p->mt;
    p->W1 = p->W;
    p->W12 = p->W;
    p->r2 = 0.0;
    p->qa = -expm1(-p->a);
    /* the GPU's lean mode without diffusion (no compat-fermion factor) */
    p->bose3 = p->boson && !cfg->compat_fermion && !cfg->include_diff;
    if (p->bose3) {
        /* term n: Gamma(3), Gamma(2), Gamma(1) at rate n with weights
         * exp(-(n-1)a) (2/n^3) (1, n m~, n^2 m~^2/4) */
        const double ea = exp(-p->a);
        p->W12 = p->W1 + 0.25 * ea * (1.0 + p->mt) * (1.0 + p->mt);
        p->W = p->W12 + (2.0 / 27.0) * ea * ea * (1.0 + 1.5 * p->mt) * (1.0 + 1.5 * p->mt);
        p->r2 = 4.0 / ea;
        p->qa = -expm1(-3.0 * p->a);
    }
    p->compat = (cfg->compat_fermion && sampler == 0) ? 1 : 0;
    p->c_poly = p->mut * p->mut - 0.5 * p->mt * p->mt;
    p->rmax = 1.0;
    if (p->compat) {
        const double amu = fabs(p->mut);
        if (p->boson) {
            p->rmax = 1.0 + (p->mut < 0 ? 4.0 * amu / (10.0 * exp(1.0) * p->mt * p->mt) : 0.0);
        } else {
            const double r = 1.0 - p->mut / p->mt;
            double C = 2.0 * r * r;
            if (C < 1.0) C = 1.0;
            const double aa = p->a > 0.1 ? p->a : 0.1;
            const double x2 = (p->a >= 0.1) ? aa * exp(-10.0 * aa) : 1.0 / (10.0 * exp(1.0));
            p->rmax = 1.0 + C * 2.0 / expm1(p->a > 1e-12 ? p->a : 1e-12)
                      + 8.0 * amu * x2 / (p->mt * p->mt);
        }
        /* the bound is attained (fermions at threshold, bosons as E -> inf):
         * a relative margin keeps rounding from crossing it */
        p->rmax *= 1.0 + 1e-5;
    }
}

/* Effective density ratio of the reference's proposal (series truncated at
 * 10 terms; fermion CDF_2 summed without its alternating sign,
 * src/FermionMomentumSampler.cpp:80-93) to the exact one. */
static double orc_compat_ratio(const orc_prop* p, double Et) {
    double S1 = 0.0, S2 = 0.0, e = 1.0;
    const double q = exp(-Et);
    for (int n = 1; n <= 10; n++) {
        e *= q;
        S2 += e;                                        /* boson series */
        S1 += (p->boson || (n & 1)) ? e : -e;           /* statistics of the table */
    }
    const double finf = p->boson ? q / (-expm1(-Et)) : q / (1.0 + q);
    const double num = Et * Et * S2 + 2.0 * p->mut * Et * S1 + p->c_poly * finf;
    const double den = (Et * Et + 2.0 * p->mut * Et + p->c_poly) * finf;
    return num / den;
}

typedef struct {
    uint32_t key[2];
    uint32_t i, e, k;
} orc_hstream;

static void orc_hblock(const orc_hstream* s, uint32_t c0, uint32_t tag, uint32_t w[4]) {
    const uint32_t ctr[4] = {c0, s->i, s->e, s->k | (tag << 16)};
    orc_philox4x32_10(ctr, s->key, w);
}

/* one proposal; returns 1 on acceptance and fills the LRF momentum */
static int orc_try(const orc_cfg* cfg, const orc_cell* c, const orc_prop* p, int sign, int B,
                   const orc_hstream* hs, uint32_t t, double* pl, double* u_rap,
                   int64_t* violations) {
    uint32_t A[4], Bw[4];
    orc_hblock(hs, 2u * t, ORC_TAG_TRY, A);
    orc_hblock(hs, 2u * t + 1u, ORC_TAG_TRY, Bw);
    const double sel = orc_u01(A[0]) * p->W;
    double prod = orc_u01_pos(A[1]);
    /* term n rescaled to weights (1, n m~, n^2 m~^2/4): Gamma(3) below 1,
     * Gamma(2) below 1 + n m~, K at rate n; the rescale is 1/2 for term 1,
     * 4 exp(a) for term 2 and 27 exp(2a) / 2 for term 3 */
    const int t2 = sel >= p->W1, t3 = sel >= p->W12;
    const double s = t3 ? (sel - p->W12) * (0.84375 * p->r2 * p->r2)
                        : (t2 ? (sel - p->W1) * p->r2 : 0.5 * sel);
    const double nt = t3 ? 3.0 : (t2 ? 2.0 : 1.0);
    if (s < 1.0 + nt * p->mt) prod *= orc_u01_pos(A[2]);
    if (s < 1.0) prod *= orc_u01_pos(A[3]);
    const double K = -log(prod) / nt;
    if (K > p->Kmax) return 0;
    const double k2 = K * (K + 2.0 * p->mt);
    const double Et = K + p->mt;                  /* E / T */
    const double ptil = sqrt(k2);                 /* |p| / T */
    const double a_pE = Et * ptil / (k2 + 0.5 * p->mt * p->mt);
    const double Etil = p->a + K;                 /* (E - mu) / T */
    const double em = exp(-Etil);
    /* bosons: f_BE / (exp(-E~) + exp(-2 E~) + exp(-3 E~)) =
     * 1 / (1 - exp(-3 E~)), at most 1 / qa */
    const double a_q = p->boson ? p->qa / (-expm1((p->bose3 ? -3.0 : -1.0) * Etil)) : 1.0 / (1.0 + em);
    double a_c = 1.0;
    if (p->compat) {
        a_c = orc_compat_ratio(p, Etil) / p->rmax;
        if (a_c > 1.0) {
            (*violations)++;
            a_c = 1.0;
        }
    }
    /* direction from the flux density max(0, d0 + beta D cos(alpha)) */
    const double d0 = fabs(c->da[0]);
    double D = sqrt(c->da[1] * c->da[1] + c->da[2] * c->da[2] + c->da[3] * c->da[3]);
    double n[3] = {0.0, 0.0, 1.0};
    if (D > 1e-30) {
        n[0] = c->da[1] / D; n[1] = c->da[2] / D; n[2] = c->da[3] / D;
    } else {
        D = 0.0;
    }
    double e1[3];
    {
        double t[3] = {0.0, 0.0, 0.0};
        if (fabs(n[2]) < 0.9) t[2] = 1.0; else t[0] = 1.0;
        double ex = t[1] * n[2] - t[2] * n[1], ey = t[2] * n[0] - t[0] * n[2];
        double ez = t[0] * n[1] - t[1] * n[0];
        const double nn = sqrt(ex * ex + ey * ey + ez * ez);
        e1[0] = ex / nn; e1[1] = ey / nn; e1[2] = ez / nn;
    }
    const double e2[3] = {n[1] * e1[2] - n[2] * e1[1], n[2] * e1[0] - n[0] * e1[2],
                          n[0] * e1[1] - n[1] * e1[0]};
    const double beta = ptil / Et;
    const double bD = beta * D;
    double c_lo = -1.0, r_flux = 1.0;
    if (bD > d0) {
        c_lo = -d0 / bD;
        r_flux = (d0 + bD) * (d0 + bD) / (beta * (d0 + D) * (d0 + D));
    } else if (D > d0) {
        r_flux = 4.0 * d0 * D / ((d0 + D) * (d0 + D));
    }
    const double a_lin = d0 + bD * c_lo;
    const double L = 1.0 - c_lo;
    const double uZ = orc_u01(Bw[0]) * (a_lin * L + 0.5 * bD * L * L);
    double cth = c_lo + 2.0 * uZ / (a_lin + sqrt(a_lin * a_lin + 2.0 * bD * uZ));
    if (cth > 1.0) cth = 1.0;
    double sth2 = 1.0 - cth * cth;
    const double sth = sth2 > 0 ? sqrt(sth2) : 0.0;
    const double phi = 2.0 * ORC_PI * (orc_u01(Bw[1]) - 0.5);   /* azimuth in [-pi, pi) */
    const double cph = cos(phi), sph = sin(phi);
    const double T = c->T;
    const double pm = T * ptil;
    const double p0 = T * Et;
    const double px = pm * (cth * n[0] + sth * (cph * e1[0] + sph * e2[0]));
    const double py = pm * (cth * n[1] + sth * (cph * e1[1] + sph * e2[1]));
    const double pz = pm * (cth * n[2] + sth * (cph * e1[2] + sph * e2[2]));
    const double f0 = em / (1.0 + sign * em);
    const double one_m = 1.0 - sign * f0;
    double df_s = 0.0, df_b = 0.0, df_q = 0.0;
    if (cfg->include_shear) {
        const double Wf = (px * px * c->pxx + 2. * px * py * c->pxy + 2. * px * pz * c->pxz
                           + py * py * c->pyy + 2. * py * pz * c->pyz
                           + pz * pz * (-c->pxx - c->pyy));
        if (cfg->neos_kind == 1) {
            df_s = one_m * Wf / (2. * c->vis2) / (p0 * T);
        } else if (cfg->neos_kind == 0) {
            df_s = one_m * Wf * c->vis0;
        } else {
            df_s = one_m * Wf / (2.0 * T * T * (c->E + c->P));
        }
    }
    if (cfg->include_bulk) {
        const int kind = cfg->bulk_kind;
        if (kind == 11) {
            df_b = one_m * c->Pi * (c->vis0 * p->m * p->m + c->vis1 * B * p0 + c->vis2 * p0 * p0);
        } else if (kind == 21 || kind == 1) {
            const double Pi = (kind == 1) ? c->Pi / ORC_HBARC : c->Pi;
            const double EoT = p0 / T;
            const double moT = p->m / T;
            df_b = -1.0 * one_m * c->vis0 * (moT * moT / (3. * EoT) - c->vis1 * EoT) * Pi;
        }
    }
    if (cfg->include_diff) {
        const double qf = (-px * c->qx - py * c->qy - pz * c->qz);
        df_q = one_m * (c->nB / (c->E + c->P) - B / p0) * qf / c->kappa;
    }
    double fact2 = (1. + df_s + df_b + df_q) / 2.;
    fact2 = fact2 < 0 ? 0 : (fact2 > 1 ? 1 : fact2);
    const double acc = a_pE * a_q * a_c * r_flux * fact2;
    if (!(orc_u01(Bw[2]) < acc)) return 0;
    pl[0] = p0; pl[1] = px; pl[2] = py; pl[3] = pz;
    *u_rap = orc_u01(Bw[3]);
    return 1;
}

static void orc_emit(const orc_cfg* cfg, const orc_cell* c, double m, int32_t pid,
                     const double* pl_d, double u_rap, orc_hadron* h) {
    /* the reference stores the LRF momentum as float before boosting */
    const float pl[4] = {(float)pl_d[0], (float)pl_d[1], (float)pl_d[2], (float)pl_d[3]};
    const double pdu = pl[1] * c->u[1] + pl[2] * c->u[2] + pl[3] * c->u[3];
    double lab[4];
    lab[0] = pl[0] * c->u[0] + pdu;
    for (int i = 1; i < 4; i++) lab[i] = pl[i] + (pdu / (c->u[0] + 1.0) + pl[0]) * c->u[i];
    const double mT2 = m * m + lab[1] * lab[1] + lab[2] * lab[2];
    const double mT = sqrt(mT2);
    double eta_s, pz, E;
    if (cfg->hydro_mode == 2) {
        eta_s = c->eta;
        pz = lab[3];
        E = sqrt(mT2 + pz * pz);
    } else {
        const double rap = cfg->y_lb + (cfg->y_rb - cfg->y_lb) * u_rap;
        const double y = asinh(lab[3] / mT);
        eta_s = rap - (y - c->eta);
        pz = mT * sinh(rap);
        E = mT * cosh(rap);
    }
    h->pid = pid;
    h->mass = (float)m;
    h->E = (float)E;
    h->px = (float)lab[1];
    h->py = (float)lab[2];
    h->pz = (float)pz;
    h->t = (float)(c->tau * cosh(eta_s));
    h->x = (float)c->xpt;
    h->y = (float)c->ypt;
    h->z = (float)(c->tau * sinh(eta_s));
}

int64_t orc_sample_replay(const orc_cfg* cfg, const orc_species* sp, int32_t n_sp,
                          const float* lrf28, int64_t n_cells, const float* coef4,
                          const uint64_t* cdf, const uint64_t* qtot, const int32_t* counts,
                          orc_hadron* out, int64_t capacity, orc_stats* stats) {
    memset(stats, 0, sizeof(*stats));
    int64_t w = 0;
    for (int64_t e = 0; e < cfg->n_events; e++) {
        const uint32_t eg = (uint32_t)(cfg->event_offset + e);
        for (int32_t k = 0; k < n_sp; k++) {
            const orc_species* s = sp + k;
            /* local_charge_conservation: two records per draw of a positive
             * species, the second a partner with opposite B, S, Q sampled in
             * the same cell (src/FSSW.cpp:1035-1048) */
            const int paired = cfg->lcc && s->charge > 0;
            const int32_t n_draws = counts[e * n_sp + k] / (paired ? 2 : 1);
            const uint64_t* row = cdf + (int64_t)k * (n_cells + 1);
            for (int32_t i = 0; i < n_draws; i++) {
                if (w + (paired ? 2 : 1) > capacity) return -1;
                orc_hstream hs;
                hs.key[0] = (uint32_t)cfg->seed;
                hs.key[1] = (uint32_t)(cfg->seed >> 32);
                hs.i = (uint32_t)i;
                hs.e = eg;
                hs.k = (uint32_t)k;
                uint32_t t = 0;
                int32_t redraw = 0;
                int done = 0;
                orc_cell c;
                while (!done) {
                    uint32_t wc[4];
                    uint64_t r;
                    if (redraw == 0) {
                        /* first cell: draws 2k and 2k + 1 share the block
                         * with counter k, halves (x, y) and (z, w) */
                        orc_hstream hp = hs;
                        hp.i = (uint32_t)i >> 1;
                        orc_hblock(&hp, 0u, ORC_TAG_CELL, wc);
                        r = (i & 1) ? (((uint64_t)wc[2] << 32) | (uint64_t)wc[3])
                                    : (((uint64_t)wc[0] << 32) | (uint64_t)wc[1]);
                    } else {
                        orc_hblock(&hs, (uint32_t)redraw, ORC_TAG_CELL, wc);
                        r = ((uint64_t)wc[0] << 32) | (uint64_t)wc[1];
                    }
                    const int64_t l = orc_search(row, n_cells, qtot[k], r);
                    orc_load_cell(lrf28, coef4, l, &c);
                    orc_prop p;
                    const double mu = s->baryon * c.muB + s->strange * c.muS + s->charge * c.muQ;
                    orc_setup(cfg, s->mass, s->sign, mu, c.T, &p);
                    if (p.status) return -2;
                    for (int32_t tr = 0; tr < cfg->max_tries; tr++) {
                        double pl[4], u_rap = 0.0;
                        const int ok = orc_try(cfg, &c, &p, s->sign, s->baryon, &hs, t, pl, &u_rap,
                                               &stats->n_bound_violations);
                        t++;
                        stats->n_tries++;
                        if (ok) {
                            orc_emit(cfg, &c, s->mass, s->pid, pl, u_rap, out + w);
                            w++;
                            done = 1;
                            break;
                        }
                    }
                    if (!done) {
                        redraw++;
                        stats->n_redraws++;
                        if (redraw > cfg->max_redraws) {
                            /* abandoned: the GPU writes empty records */
                            for (int q = 0; q < (paired ? 2 : 1); q++) {
                                memset(out + w, 0, sizeof(orc_hadron));
                                w++;
                                stats->n_failures++;
                            }
                            done = 2;
                        }
                    }
                }
                if (!paired || done == 2) continue;
                /* the partner: same cell and mass, opposite quantum numbers; the
                 * proposal counter t continues and the cell is never redrawn */
                orc_prop p2;
                const double mu2 =
                    (-s->baryon) * c.muB + (-s->strange) * c.muS + (-s->charge) * c.muQ;
                orc_setup(cfg, s->mass, s->sign, mu2, c.T, &p2);
                if (p2.status) return -2;
                int pdone = 0;
                while (!pdone) {
                    for (int32_t tr = 0; tr < cfg->max_tries; tr++) {
                        double pl[4], u_rap = 0.0;
                        const int ok = orc_try(cfg, &c, &p2, s->sign, -s->baryon, &hs, t, pl,
                                               &u_rap, &stats->n_bound_violations);
                        t++;
                        stats->n_tries++;
                        if (ok) {
                            orc_emit(cfg, &c, s->mass, -s->pid, pl, u_rap, out + w);
                            w++;
                            pdone = 1;
                            break;
                        }
                    }
                    if (!pdone) {
                        redraw++;
                        stats->n_redraws++;
                        if (redraw > cfg->max_redraws) {
                            memset(out + w, 0, sizeof(orc_hadron));
                            w++;
                            stats->n_failures++;
                            pdone = 1;
                        }
                    }
                }
            }
        }
    }
    return w;
}


