/* Test infrastructure only -- oracle part 3: the reference's own sampling
 * algorithm restated in C, used as the timed CPU baseline and as an
 * independent statistical check of the GPU sampler.
 *
 * It follows, step for step:
 *   FSSW::sample_using_dN_dxtdy_4all_particles_conventional, src/FSSW.cpp:873-1071
 *     (per species: yields, FP64 CDF, per event a Poisson count, per hadron a
 *      binary search over the CDF, coefficient lookups, momentum, record)
 *   FSSW::determine_number_to_sample (model 30), src/FSSW.cpp:293-297
 *   RandomVariable1DArray::rand, src/RandomVariable1DArray.cpp:67-70 and
 *     binarySearch, src/arsenal.cpp:644-678
 *   FSSW::sample_momemtum_from_a_fluid_cell, src/FSSW.cpp:1852-1966
 *   MomentumSamplerShell::Sample_a_momentum, src/MomentumSamplerShell.cpp:24-48
 *   MomentumSamplerBase::Sample_a_momentum / inverse_CDF, src/MomentumSamplerBase.cpp:20-93
 *   Boson/FermionMomentumSampler tables and CDF_0/1/2 series,
 *     src/BosonMomentumSampler.cpp:7-87, src/FermionMomentumSampler.cpp:8-93
 *     (including the fermion CDF_2 summed without its alternating sign)
 *   FSSW::add_one_sampled_particle / boost, src/FSSW.cpp:1969-2010
 * The uniforms come from a 32-bit Mersenne twister (MT19937, Matsumoto &
 * Nishimura 1998) combined two draws per double, as std::mt19937 with
 * std::uniform_real_distribution<double> does in the reference
 * (src/Random.h:11-22); Poisson counts use Hormann's PTRS. */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "oracle.h"

/* ---------------------------------------------------------------- MT19937 */
typedef struct {
    uint32_t mt[624];
    int idx;
} orc_mt;

static void mt_seed(orc_mt* s, uint32_t seed) {
    s->mt[0] = seed;
    for (int i = 1; i < 624; i++)
        s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
    s->idx = 624;
}

static uint32_t mt_next(orc_mt* s) {
    if (s->idx >= 624) {
        for (int i = 0; i < 624; i++) {
            const uint32_t y = (s->mt[i] & 0x80000000u) | (s->mt[(i + 1) % 624] & 0x7fffffffu);
            uint32_t v = s->mt[(i + 397) % 624] ^ (y >> 1);
            if (y & 1u) v ^= 0x9908b0dfu;
            s->mt[i] = v;
        }
        s->idx = 0;
    }
    uint32_t y = s->mt[s->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

static double mt_uniform(orc_mt* s) {
    const double a = mt_next(s);
    const double b = mt_next(s);
    double r = (a + b * 4294967296.0) / 18446744073709551616.0;
    if (r >= 1.0) r = 0.99999999999999989;
    return r;
}

/* ------------------------------------------------- momentum samplers (6) */
typedef struct {
    int fermion;
    double m0;
    int trunc;
    int len;
    double* E;
    double* C0;
    double* C1;
    double* C2;
    double cache_a, c0a, c1a, c2a;
} orc_psampler;

static double cdf_k(const orc_psampler* p, int k, double Et) {
    const double m = p->m0;
    double res = 0.0;
    if (k == 0 && p->trunc > 5) {
        return p->fermion ? -exp(m) * log((1. + exp(-Et)) / (1. + exp(-m)))
                          : exp(m) * log((1. - exp(-Et)) / (1. - exp(-m)));
    }
    double sign = 1.0;
    for (int n = 0; n < p->trunc; n++) {
        const double n1 = n + 1;
        double term;
        if (k == 0) {
            /* the fermion series divides two ints (sign/n1), so only its
             * first term survives; the boson series divides doubles */
            const double w = p->fermion ? (n == 0 ? 1.0 : 0.0) : 1. / n1;
            term = w * exp(-m * n) * (1. - exp((m - Et) * n1));
        } else if (k == 1) {
            term = 1. / (n1 * n1) * exp(-m * n) * ((m * n1 + 1) - exp((m - Et) * n1) * (Et * n1 + 1));
        } else {
            term = 1. / (n1 * n1 * n1) * exp(-m * n) *
                   ((m * n1 * (m * n1 + 2) + 2) - exp((m - Et) * n1) * (Et * n1 * (Et * n1 + 2) + 2));
        }
        /* the fermion CDF_2 series carries no alternating sign (reference) */
        if (p->fermion && k != 2) term *= sign;
        res += term;
        sign = -sign;
    }
    return res;
}

static void psampler_init(orc_psampler* p, int fermion, double m0, int trunc) {
    p->fermion = fermion;
    p->m0 = m0;
    p->trunc = trunc;
    const double emin = fermion ? m0 : m0 + 0.05;
    const double span = fermion ? 40. : 50.;
    const double de = fermion ? 0.02 : 0.05;
    p->len = (int)(span / de + 1);
    p->E = (double*)malloc(sizeof(double) * (size_t)p->len);
    p->C0 = (double*)malloc(sizeof(double) * (size_t)p->len);
    p->C1 = (double*)malloc(sizeof(double) * (size_t)p->len);
    p->C2 = (double*)malloc(sizeof(double) * (size_t)p->len);
    for (int i = 0; i < p->len; i++) {
        const double e = emin + i * de;
        p->E[i] = e;
        p->C0[i] = cdf_k(p, 0, e);
        p->C1[i] = cdf_k(p, 1, e);
        p->C2[i] = cdf_k(p, 2, e);
    }
    p->cache_a = 1.0;
    p->c0a = cdf_k(p, 0, 1.0);
    p->c1a = cdf_k(p, 1, 1.0);
    p->c2a = cdf_k(p, 2, 1.0);
}

static void psampler_free(orc_psampler* p) {
    free(p->E); free(p->C0); free(p->C1); free(p->C2);
}

static double inverse_cdf(const orc_psampler* p, double r, int idx0, double rmax_in, double mterm,
                          double mt, double mut) {
    int lo = idx0, hi = p->len - 1;
    const double c = mut * mut - mt * mt / 2.;
    double rmin = p->C2[lo] + 2. * mut * p->C1[lo] + c * p->C0[lo] - mterm;
    double rmax = rmax_in;
    while (hi - lo > 1) {
        const int mid = (int)((hi + lo) / 2 + 0.1);
        const double rm = p->C2[mid] + 2. * mut * p->C1[mid] + c * p->C0[mid] - mterm;
        if (r < rm) { hi = mid; rmax = rm; } else { lo = mid; rmin = rm; }
    }
    double E0 = p->E[lo];
    if (E0 < mt - mut) {
        E0 = mt - mut;
        rmin = 0.;
    }
    const double d = (rmax - rmin) > 1e-16 ? (rmax - rmin) : 1e-16;
    return E0 + (p->E[hi] - E0) / d * (r - rmin);
}

/* returns |p|, or -1 when m/T - mu/T is off the table */
static double psampler_draw(orc_psampler* p, orc_mt* rng, double m, double T, double mu) {
    if (T < 1e-16) T = 1e-16;
    const double mt = m / T, mut = mu / T;
    const double a = mt - mut;
    if (fabs(a - p->cache_a) > 1e-8) {
        p->cache_a = a;
        p->c0a = cdf_k(p, 0, a);
        p->c1a = cdf_k(p, 1, a);
        p->c2a = cdf_k(p, 2, a);
    }
    const double c = mut * mut - mt * mt / 2.;
    const double mterm = p->c2a + 2. * mut * p->c1a + c * p->c0a;
    const int last = p->len - 1;
    const double cmax = p->C2[last] + 2. * mut * p->C1[last] + c * p->C0[last] - mterm;
    const int idx_min = (int)((a - p->E[0]) / (p->E[1] - p->E[0]));
    if (idx_min < 0 || idx_min >= last) return -1.0;
    double ps, acc;
    do {
        const double r = mt_uniform(rng) * cmax;
        const double et = inverse_cdf(p, r, idx_min, cmax, mterm, mt, mut);
        const double E = T * et + mu;
        ps = sqrt(E * E - m * m);
        acc = (ps / E) / (1. - m * m / (2. * E * E));
    } while (mt_uniform(rng) > acc);
    return ps;
}

typedef struct {
    orc_psampler b[3], f[3];
} orc_shell;

static void shell_init(orc_shell* s) {
    psampler_init(&s->f[0], 1, 0.0, 10);
    psampler_init(&s->f[1], 1, 30.0, 2);
    psampler_init(&s->f[2], 1, 50.0, 1);
    psampler_init(&s->b[0], 0, 0.05, 10);
    psampler_init(&s->b[1], 0, 30.0, 2);
    psampler_init(&s->b[2], 0, 50.0, 1);
}

static void shell_free(orc_shell* s) {
    for (int i = 0; i < 3; i++) { psampler_free(&s->b[i]); psampler_free(&s->f[i]); }
}

static double shell_draw(orc_shell* s, orc_mt* rng, double m, double T, double mu, int sign) {
    const double a = m / T - mu / T;
    const int k = a < 30. ? 0 : (a < 50. ? 1 : 2);
    return (sign == -1) ? psampler_draw(&s->b[k], rng, m, T, mu)
                        : psampler_draw(&s->f[k], rng, m, T, mu);
}

/* ----------------------------------------------------- helpers from part 1 */
/* (re-stated here: part 1 keeps them file-local) */
static void ref_bulk14(const orc_cfg* c, double T, double muB, double* out) {
    const int idx_T = (int)((T - c->b14_T0) / c->b14_dT);
    const int idx_mu = (int)((muB - c->b14_mu0) / c->b14_dmu);
    const double xf = ((T - c->b14_T0) / c->b14_dT - idx_T);
    const double yf = ((muB - c->b14_mu0) / c->b14_dmu - idx_mu);
    const int nT = c->b14_nT, nmu = c->b14_nmu;
    const int iT1 = idx_T < 0 ? 0 : (idx_T > nT - 1 ? nT - 1 : idx_T);
    const int iT2 = idx_T + 1 < 0 ? 0 : (idx_T + 1 > nT - 1 ? nT - 1 : idx_T + 1);
    const int im1 = idx_mu < 0 ? 0 : (idx_mu > nmu - 1 ? nmu - 1 : idx_mu);
    const int im2 = idx_mu + 1 < 0 ? 0 : (idx_mu + 1 > nmu - 1 ? nmu - 1 : idx_mu + 1);
    const double* tabs[3] = {c->b14_c0, c->b14_c1, c->b14_c2};
    double v[3];
    for (int k = 0; k < 3; k++) {
        const double* tb = tabs[k];
        v[k] = (tb[iT1 * nmu + im1] * (1. - xf) * (1. - yf) + tb[iT1 * nmu + im2] * (1. - xf) * yf +
                tb[iT2 * nmu + im2] * xf * yf + tb[iT2 * nmu + im1] * xf * (1. - yf));
    }
    const double T3 = T * T * T, T4 = T3 * T;
    out[0] = (v[0] - v[2]) / T4;
    out[1] = v[1] / T3;
    out[2] = (4. * v[2] - v[0]) / T4;
}

static int64_t ref_poisson(orc_mt* rng, double mu) {
    if (mu < 12.0) {
        const double u = mt_uniform(rng);
        double p = exp(-mu), cdf = p;
        int64_t k = 0;
        while (u > cdf && k < 100000) { k++; p *= mu / (double)k; cdf += p; }
        return k;
    }
    const double smu = sqrt(mu), b = 0.931 + 2.53 * smu, a = -0.059 + 0.02483 * b;
    const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2.0);
    const double log_mu = log(mu);
    for (;;) {
        const double U = mt_uniform(rng) - 0.5, V = mt_uniform(rng);
        const double us = 0.5 - fabs(U);
        const double kd = floor((2.0 * a / us + b) * U + mu + 0.43);
        if (us >= 0.07 && V <= vr) return (int64_t)kd;
        if (kd < 0.0 || (us < 0.013 && V > us)) continue;
        if (log(V) + log(inv_alpha) - log(a / (us * us) + b) <= -mu + kd * log_mu - lgamma(kd + 1.0))
            return (int64_t)kd;
    }
}

static int64_t ref_search(const double* cdf, int64_t len, double v) {
    int64_t i = 0, f = len - 1;
    if (v > cdf[f]) return len - 1;
    if (v < cdf[0]) return -1;
    int64_t idx = (f + i) / 2;
    while (f - i > 1) {
        if (cdf[idx] < v) i = idx; else f = idx;
        idx = (f + i) / 2;
    }
    return i;
}

/* --------------------------------------------------------------- sampler */
int64_t orc_reference_sampler(const orc_cfg* c, const orc_species* sp, int32_t n_sp,
                              const float* lrf28, const int32_t* keep, int64_t n_cells,
                              int32_t n_threads, uint64_t seed, orc_hadron* out,
                              int64_t capacity, double* seconds) {
    (void)n_threads;
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    orc_mt rng;
    mt_seed(&rng, (uint32_t)seed);
    orc_shell shell;
    shell_init(&shell);
    double* y = (double*)malloc(sizeof(double) * (size_t)n_cells);
    double* cdf = (double*)malloc(sizeof(double) * (size_t)(n_cells + 1));
    int64_t written = 0;
    const double ymult = (c->hydro_mode != 2) ? (c->y_rb - c->y_lb) : 1.0;
    const int neos = c->neos_kind;
    for (int32_t k = 0; k < n_sp; k++) {
        const orc_species* p = sp + k;
        /* yields of this species (the reference recomputes them per species) */
        if (orc_yields(c, p, 1, lrf28, keep, n_cells, y) != 0) { written = -3; goto done; }
        double sum = 0.0;
        cdf[0] = 0.0;
        for (int64_t l = 0; l < n_cells; l++) {
            sum += y[l] > 0 ? y[l] : 0;
            cdf[l + 1] = sum;
        }
        const double dN = ymult * sum;
        const double m = p->mass;
        for (int64_t e = 0; e < c->n_events; e++) {
            const int64_t nsamp = dN < 1e-15 ? 0 : ref_poisson(&rng, dN);
            int64_t got = 0;
            while (got < nsamp) {
                const int64_t l = ref_search(cdf, n_cells + 1,
                                             cdf[0] + (sum - cdf[0] - 1e-15) * mt_uniform(&rng));
                const float* s = lrf28 + 28 * l;
                const double T = s[13], muB = s[16];
                double vis[3] = {0, 0, 0};
                double kappa = 1.0;
                /* per-hadron coefficient lookups as in src/FSSW.cpp:982-1008 */
                if (c->include_bulk && neos == -1 && c->bulk_kind == 11) ref_bulk14(c, T, muB, vis);
                double cc[4];
                if (neos == 1 || c->include_diff) {
                    orc_cell_coeffs(c, s, 1, cc);
                    if (neos == 1) { vis[0] = cc[0]; vis[1] = cc[1]; vis[2] = cc[2]; }
                    if (c->include_diff) kappa = cc[3];
                }
                /* sample_momemtum_from_a_fluid_cell */
                double mu = p->baryon * s[16] + p->strange * s[17] + p->charge * s[18];
                if (mu > m) mu = m;
                const double pref = 1.0 / (2.0 * T * T * ((double)s[12] + (double)s[14]));
                const double pref_q = (double)s[15] / ((double)s[12] + (double)s[14]);
                const double dsfac = fabs((double)s[4]) + sqrt((double)s[5] * s[5] + (double)s[6] * s[6] +
                                                               (double)s[7] * s[7]);
                int ok = 0;
                double pl[4];
                for (int tries = 1; tries < 5000; tries++) {
                    const double pm = shell_draw(&shell, &rng, m, T, mu, p->sign);
                    if (pm < 0) { written = -2; goto done; }
                    const double phi = 2 * 3.14159265358979323846 * mt_uniform(&rng);
                    const double cth = 2. * mt_uniform(&rng) - 1.;
                    const double sth = sqrt(1. - cth * cth);
                    const double px = pm * sth * cos(phi), py = pm * sth * sin(phi), pz = pm * cth;
                    const double p0 = sqrt(m * m + pm * pm);
                    const double pds = p0 * s[4] + px * s[5] + py * s[6] + pz * s[7];
                    const double f0 = 1. / (exp((p0 - mu) / T) + p->sign);
                    const double om = 1. - p->sign * f0;
                    double dfs = 0., dfb = 0., dfq = 0.;
                    if (c->include_shear) {
                        const double W = px * px * s[20] + 2. * px * py * s[21] + 2. * px * pz * s[22] +
                                         py * py * s[23] + 2. * py * pz * s[24] + pz * pz * (-s[20] - s[23]);
                        if (neos == 1) dfs = om * W / (2. * vis[2]) / (p0 * T);
                        else if (neos == 0) dfs = om * W * vis[0];
                        else dfs = om * W * pref;
                    }
                    if (c->include_bulk) {
                        if (c->bulk_kind == 11) {
                            dfb = om * s[19] * (vis[0] * m * m + vis[1] * p->baryon * p0 + vis[2] * p0 * p0);
                        } else if (c->bulk_kind == 21 || c->bulk_kind == 1) {
                            const double Pi = c->bulk_kind == 1 ? s[19] / ORC_HBARC : s[19];
                            const double EoT = p0 / T, moT = m / T;
                            dfb = -om * vis[0] * (moT * moT / (3. * EoT) - vis[1] * EoT) * Pi;
                        }
                    }
                    if (c->include_diff) {
                        const double qf = -px * s[25] - py * s[26] - pz * s[27];
                        dfq = om * (pref_q - p->baryon / p0) * qf / kappa;
                    }
                    double f1 = pds / p0 / dsfac, f2 = (1. + dfs + dfb + dfq) / 2.;
                    f1 = f1 < 0 ? 0 : (f1 > 1 ? 1 : f1);
                    f2 = f2 < 0 ? 0 : (f2 > 1 ? 1 : f2);
                    if (mt_uniform(&rng) < f1 * f2) {
                        pl[0] = p0; pl[1] = px; pl[2] = py; pl[3] = pz;
                        ok = 1;
                        break;
                    }
                }
                if (!ok) continue;   /* the reference redraws the cell */
                got++;
                /* boost (float 4-vectors as in the reference) and record */
                const float pf[4] = {(float)pl[0], (float)pl[1], (float)pl[2], (float)pl[3]};
                const double u0 = s[8], u1 = s[9], u2 = s[10], u3 = s[11];
                const double pdu = pf[1] * u1 + pf[2] * u2 + pf[3] * u3;
                const float lab1 = (float)(pf[1] + (pdu / (u0 + 1) + pf[0]) * u1);
                const float lab2 = (float)(pf[2] + (pdu / (u0 + 1) + pf[0]) * u2);
                const float lab3 = (float)(pf[3] + (pdu / (u0 + 1) + pf[0]) * u3);
                const double pT = sqrt((double)lab1 * lab1 + (double)lab2 * lab2);
                const double ph = atan2(lab2, lab1);
                const double mT = sqrt(pT * pT + m * m);
                const double yv = asinh(lab3 / mT);
                const double ymes = yv - s[3];
                double eta_s = s[3];
                if (c->hydro_mode != 2) eta_s = (c->y_lb + (c->y_rb - c->y_lb) * mt_uniform(&rng)) - ymes;
                const double rap = ymes + eta_s;
                if (out && written < capacity) {
                    orc_hadron* h = out + written;
                    h->pid = p->pid;
                    h->mass = (float)m;
                    h->px = (float)(pT * cos(ph));
                    h->py = (float)(pT * sin(ph));
                    h->pz = (float)(mT * sinh(rap));
                    h->E = (float)(mT * cosh(rap));
                    h->t = (float)(s[0] * cosh(eta_s));
                    h->x = s[1];
                    h->y = s[2];
                    h->z = (float)(s[0] * sinh(eta_s));
                }
                written++;
            }
        }
    }
done:
    free(y);
    free(cdf);
    shell_free(&shell);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (seconds) *seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
    return written;
}
