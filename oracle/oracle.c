/* Test infrastructure only -- oracle part 1 (direct FP64 restatement of the
 * reference's per-cell work) and part 2a (per (event, species) counts on the
 * Philox streams of the GPU sampler).  See oracle.h. */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "philox.h"

/* GSL-compatible special functions, oracle/gsl_compat/gsl_compat.cpp */
double gsl_sf_bessel_K1(double x);
double gsl_sf_bessel_Kn(int n, double x);
double gsl_sf_expint_E2(double x);
double gsl_sf_expint_En(int n, double x);

/* ------------------------------------------------------------------------ */
/* special-function tables: FSSW::initialize_special_function_arrays,
 * src/FSSW.cpp:1609-1643 */
void orc_sf_tables(int include_bulk, int include_diff, double* sf_K, double* sf_E) {
    for (int i = 0; i < ORC_SF_LEN; i++) {
        const double x = ORC_SF_X0 + i * ORC_SF_DX;
        sf_K[3 * i + 0] = include_bulk ? gsl_sf_bessel_K1(x) : 0.0;
        sf_K[3 * i + 1] = gsl_sf_bessel_Kn(2, x);
        sf_K[3 * i + 2] = include_bulk ? gsl_sf_bessel_Kn(3, x) : 0.0;
        if (include_diff && sf_E) {
            sf_E[ORC_N_EXPINT * i + 0] = gsl_sf_expint_E2(x);
            for (int k = 1; k < ORC_N_EXPINT; k++) {
                sf_E[ORC_N_EXPINT * i + k] = gsl_sf_expint_En(2 * k + 2, x);
            }
        }
    }
}

/* get_special_function_K1/K2/K3, src/FSSW.cpp:1646-1703: linear
 * interpolation on the table, direct evaluation off the table */
double orc_sf_K(const orc_cfg* c, int which, double arg) {
    if (arg < ORC_SF_X0 || arg > ORC_SF_XMAX - ORC_SF_DX) {
        return which == 1 ? gsl_sf_bessel_K1(arg) : gsl_sf_bessel_Kn(which, arg);
    }
    const int idx = (int)((arg - ORC_SF_X0) / ORC_SF_DX);
    const double fraction = (arg - ORC_SF_X0 - idx * ORC_SF_DX) / ORC_SF_DX;
    return (1. - fraction) * c->sf_K[3 * idx + which - 1]
           + fraction * c->sf_K[3 * (idx + 1) + which - 1];
}

/* get_special_function_En, src/FSSW.cpp:1706-1727 */
static void orc_sf_En(const orc_cfg* c, double arg, double* res) {
    if (arg < ORC_SF_X0 || arg > ORC_SF_XMAX - ORC_SF_DX) {
        res[0] = gsl_sf_expint_E2(arg);
        for (int i = 1; i < ORC_N_EXPINT; i++) res[i] = gsl_sf_expint_En(2 * i + 2, arg);
        return;
    }
    const int idx = (int)((arg - ORC_SF_X0) / ORC_SF_DX);
    const double fraction = (arg - ORC_SF_X0 - idx * ORC_SF_DX) / ORC_SF_DX;
    for (int i = 0; i < ORC_N_EXPINT; i++) {
        res[i] = (1. - fraction) * c->sf_E[ORC_N_EXPINT * idx + i]
                 + fraction * c->sf_E[ORC_N_EXPINT * (idx + 1) + i];
    }
}

/* ------------------------------------------------------------------------ */
/* regulate_surface_cells (src/readindata.cpp:768-842, regulate_Wmunu
 * :1216-1246) followed by iSS::transform_to_local_rest_frame
 * (src/iSS.cpp:170-293).  The float/double mix of the reference is kept
 * (float members, double temporaries) so the LRF cells agree bit for bit.
 * Input rows follow FO_surf (34 floats), output rows FO_surf_LRF (28 floats). */
void orc_lrf_cells(const float* fo34, int64_t n, float* lrf28, int32_t* keep) {
    for (int64_t l = 0; l < n; l++) {
        const float* s = fo34 + 34 * l;
        float tau = s[0], xpt = s[1], ypt = s[2], eta = s[3];
        float da0 = s[4], da1 = s[5], da2 = s[6], da3 = s[7];
        float u0 = s[8], u1 = s[9], u2 = s[10], u3 = s[11];
        float Edec = s[12], Tdec = s[13], Pdec = s[14], Bn = s[15];
        float muB = s[16], muS = s[17], muQ = s[18];
        float pi[10];
        for (int k = 0; k < 10; k++) pi[k] = s[19 + k];
        float bulkPi = s[29];
        float q0 = s[30], q1 = s[31], q2 = s[32], q3 = s[33];
        (void)q0;

        /* regulation */
        u0 = (float)sqrt(1. + u1 * u1 + u2 * u2 + u3 * u3);
        q0 = ((u1 * q1 + u2 * q2 + u3 * q3) / u0);
        {
            const double g[4] = {-1., 1., 1., 1.};
            double u[4] = {u0, u1, u2, u3};
            double W[4][4] = {{pi[0], pi[1], pi[2], pi[3]},
                              {pi[1], pi[4], pi[5], pi[6]},
                              {pi[2], pi[5], pi[7], pi[8]},
                              {pi[3], pi[6], pi[8], pi[9]}};
            double udp[4], umu[4];
            for (int i = 0; i < 4; i++) {
                udp[i] = (-u[0] * W[0][i] + u[1] * W[1][i] + u[2] * W[2][i] + u[3] * W[3][i]);
                umu[i] = g[i] * u[i];
            }
            const double tr = -W[0][0] + W[1][1] + W[2][2] + W[3][3];
            double udpdu = 0.0;
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++) udpdu += umu[i] * W[i][j] * umu[j];
            double R[4][4];
            for (int i = 0; i < 4; i++) {
                for (int j = 0; j < 4; j++) {
                    const double gij = (i == j) ? g[i] : 0.0;
                    R[i][j] = (W[i][j] + u[i] * udp[j] + u[j] * udp[i] + u[i] * u[j] * udpdu
                               - 1. / 3. * (gij + u[i] * u[j]) * (tr + udpdu));
                }
            }
            pi[0] = (float)R[0][0]; pi[1] = (float)R[0][1]; pi[2] = (float)R[0][2];
            pi[3] = (float)R[0][3]; pi[4] = (float)R[1][1]; pi[5] = (float)R[1][2];
            pi[6] = (float)R[1][3]; pi[7] = (float)R[2][2]; pi[8] = (float)R[2][3];
            pi[9] = (float)R[3][3];
        }

        /* local rest frame */
        float* o = lrf28 + 28 * l;
        const float ch = (float)cosh(eta);
        const float sh = (float)sinh(eta);
        const float ut = u0 * ch + u3 * sh;
        const float uz = u3 * ch + u0 * sh;
        const float ux = u1;
        const float uy = u2;
        const double L[4][4] = {
            {ut, -ux, -uy, -uz},
            {-ux, 1. + ux * ux / (ut + 1.), ux * uy / (ut + 1.), ux * uz / (ut + 1.)},
            {-uy, ux * uy / (ut + 1.), 1. + uy * uy / (ut + 1.), uy * uz / (ut + 1.)},
            {-uz, ux * uz / (ut + 1.), uy * uz / (ut + 1.), 1. + uz * uz / (ut + 1.)}};
        const float da_up[4] = {tau * da0 * ch - da3 * sh, -tau * da1, -tau * da2,
                                -da3 * ch + tau * da0 * sh};
        float da_lrf[4] = {0.f, 0.f, 0.f, 0.f};
        float da_mu[4];
        for (int i = 0; i < 4; i++) {
            for (int j = 0; j < 4; j++) da_lrf[i] += L[i][j] * da_up[j];
            da_mu[i] = (i == 0) ? da_lrf[i] : -da_lrf[i];
        }
        keep[l] = (da_mu[0] < 0) ? 0 : 1;
        const float q_tz[4] = {q0 * ch + q3 * sh, q1, q2, q3 * ch + q0 * sh};
        float q_lrf[4] = {0.f, 0.f, 0.f, 0.f};
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) q_lrf[i] += L[i][j] * q_tz[j];
        float pt[4][4];
        pt[0][0] = (pi[0] * ch * ch + 2. * pi[3] * ch * sh + pi[9] * sh * sh);
        pt[0][1] = pi[1] * ch + pi[6] * sh;
        pt[0][2] = pi[2] * ch + pi[8] * sh;
        pt[0][3] = (pi[0] * ch * sh + pi[3] * (ch * ch + sh * sh) + pi[9] * sh * ch);
        pt[1][0] = pt[0][1];
        pt[1][1] = pi[4];
        pt[1][2] = pi[5];
        pt[1][3] = pi[1] * sh + pi[6] * ch;
        pt[2][0] = pt[0][2];
        pt[2][1] = pi[5];
        pt[2][2] = pi[7];
        pt[2][3] = pi[2] * sh + pi[8] * ch;
        pt[3][0] = pt[0][3];
        pt[3][1] = pt[1][3];
        pt[3][2] = pt[2][3];
        pt[3][3] = (pi[0] * sh * sh + 2. * pi[3] * sh * ch + pi[9] * ch * ch);
        float pl[4][4];
        for (int i = 0; i < 4; i++) {
            for (int j = 0; j < 4; j++) {
                pl[i][j] = 0.f;
                for (int a = 0; a < 4; a++)
                    for (int b = 0; b < 4; b++) pl[i][j] += (L[i][a] * pt[a][b] * L[b][j]);
            }
        }
        o[0] = tau; o[1] = xpt; o[2] = ypt; o[3] = eta;
        o[4] = da_mu[0]; o[5] = da_mu[1]; o[6] = da_mu[2]; o[7] = da_mu[3];
        o[8] = ut; o[9] = ux; o[10] = uy; o[11] = uz;
        o[12] = Edec; o[13] = Tdec; o[14] = Pdec; o[15] = Bn;
        o[16] = muB; o[17] = muS; o[18] = muQ; o[19] = bulkPi;
        o[20] = pl[1][1]; o[21] = pl[1][2]; o[22] = pl[1][3]; o[23] = pl[2][2]; o[24] = pl[2][3];
        o[25] = q_lrf[1]; o[26] = q_lrf[2]; o[27] = q_lrf[3];
    }
}

/* ------------------------------------------------------------------------ */
/* delta-f coefficient lookups */

/* FSSW::getbulkvisCoefficients(T, muB), src/FSSW.cpp:1379-1430 */
static void orc_bulk14(const orc_cfg* c, double T, double muB, double* out) {
    const int idx_T = (int)((T - c->b14_T0) / c->b14_dT);
    const int idx_mu = (int)((muB - c->b14_mu0) / c->b14_dmu);
    const double xf = ((T - c->b14_T0) / c->b14_dT - idx_T);
    const double yf = ((muB - c->b14_mu0) / c->b14_dmu - idx_mu);
    const int nT = c->b14_nT, nmu = c->b14_nmu;
#define ORC_CLAMP(v, hi) ((v) < 0 ? 0 : ((v) > (hi) ? (hi) : (v)))
    const int iT1 = ORC_CLAMP(idx_T, nT - 1), iT2 = ORC_CLAMP(idx_T + 1, nT - 1);
    const int im1 = ORC_CLAMP(idx_mu, nmu - 1), im2 = ORC_CLAMP(idx_mu + 1, nmu - 1);
#undef ORC_CLAMP
    const double* tabs[3] = {c->b14_c0, c->b14_c1, c->b14_c2};
    double v[3];
    for (int k = 0; k < 3; k++) {
        const double* tb = tabs[k];
        const double f1 = tb[iT1 * nmu + im1], f2 = tb[iT1 * nmu + im2];
        const double f3 = tb[iT2 * nmu + im2], f4 = tb[iT2 * nmu + im1];
        v[k] = (f1 * (1. - xf) * (1. - yf) + f2 * (1. - xf) * yf + f3 * xf * yf
                + f4 * xf * (1. - yf));
    }
    const double T3 = T * T * T;
    const double T4 = T3 * T;
    out[0] = (v[0] - v[2]) / T4;
    out[1] = v[1] / T3;
    out[2] = (4. * v[2] - v[0]) / T4;
}

/* FSSW::getbulkvisCoefficients(T) for bulk_deltaf_kind == 1,
 * src/FSSW.cpp:1109-1136 (polynomial fits in T [1/fm]) */
static void orc_bulk_rta(double T, double* out) {
    static const double a[11] = {642096.624265727, -8163329.49562861, 47162768.4292073,
                                 -162590040.002683, 369637951.096896, -578181331.809836,
                                 629434830.225675, -470493661.096657, 230936465.421,
                                 -67175218.4629078, 8789472.32652964};
    static const double b[11] = {1.18171174036192, -17.6740645873717, 136.298469057177,
                                 -635.999435106846, 1918.77100633321, -3836.32258307711,
                                 5136.35746882372, -4566.22991441914, 2593.45375240886,
                                 -853.908199724349, 124.260460450113};
    const double x = T / ORC_HBARC;
    double p[11];
    p[1] = x;
    for (int k = 2; k < 11; k++) p[k] = p[k - 1] * x;
    double s0 = a[0], s1 = b[0];
    for (int k = 1; k < 11; k++) {
        s0 += a[k] * p[k];
        s1 += b[k] * p[k];
    }
    out[0] = s0;
    out[1] = s1;
    out[2] = 0.0;
}

/* FSSW::getCENEOSBQSCoefficients, src/FSSW.cpp:1433-1487 */
static void orc_ce_neos(const orc_cfg* c, double Edec, double nB, double* out) {
    const double* tb = c->ce_tb;
    const int ne = 200, nnb = 200;
    const double de = tb[5 * 200 + 0] - tb[0];
    int idx_e = (int)((Edec - tb[0]) / de);
    if (idx_e > ne - 2) idx_e = ne - 2;
    if (idx_e < 0) idx_e = 0;
    const int Ne1 = idx_e * ne;
    const int Ne2 = (idx_e + 1) * ne;
    const double e_frac = ((Edec - tb[5 * Ne1]) / de);
    const double dnB1 = tb[5 * (Ne1 + 1) + 1];
    const double dnB2 = tb[5 * (Ne2 + 1) + 1];
    int i1 = (int)(nB / dnB1);
    int i2 = (int)(nB / dnB2);
    if (i1 > nnb - 2) i1 = nnb - 2;
    if (i2 > nnb - 2) i2 = nnb - 2;
    double f1 = (nB - tb[5 * (Ne1 + i1) + 1]) / dnB1;
    double f2 = (nB - tb[5 * (Ne2 + i2) + 1]) / dnB2;
    if (f1 > 1.) f1 = 1.;
    if (f2 > 1.) f2 = 1.;
    double coef[3];
    for (int i = 2; i < 5; i++) {
        const double t1 = tb[5 * (Ne1 + i1) + i] * (1 - f1) + tb[5 * (Ne1 + i1 + 1) + i] * f1;
        const double t2 = tb[5 * (Ne2 + i2) + i] * (1 - f2) + tb[5 * (Ne2 + i2 + 1) + i] * f2;
        coef[i - 2] = t1 * (1. - e_frac) + t2 * e_frac;
    }
    out[0] = 1. / coef[1];
    out[1] = 1. / 3. - coef[0];
    out[2] = coef[2];
}

/* FSSW::get_deltaf_qmu_coeff, src/FSSW.cpp:1571-1606 */
static double orc_qmu_coeff(const orc_cfg* c, double T, double muB) {
    const double T0 = 0.05, mu0 = 0.0, dT = 0.001, dmu = 0.007892;
    const int nT = 150, nmu = 100;
    const int idx_T = (int)((T - T0) / dT);
    const int idx_mu = (int)((muB - mu0) / dmu);
    const double xf = ((T - T0) / dT - idx_T);
    const double yf = ((muB - mu0) / dmu - idx_mu);
    if (idx_mu > nmu - 2 || idx_T > nT - 2 || idx_mu < 0 || idx_T < 0) return 1e30;
    const double* tb = c->qmu_tb;
    const double f1 = tb[idx_T * nmu + idx_mu], f2 = tb[idx_T * nmu + idx_mu + 1];
    const double f3 = tb[(idx_T + 1) * nmu + idx_mu + 1], f4 = tb[(idx_T + 1) * nmu + idx_mu];
    return (f1 * (1. - xf) * (1. - yf) + f2 * (1. - xf) * yf + f3 * xf * yf
            + f4 * xf * (1. - yf));
}

/* The per-cell coefficients the sampler and the yields use:
 * coef4 = {vis0, vis1, vis2, kappa_B}. */
static void orc_cell_coeff_one(const orc_cfg* c, const float* cell, double* coef4) {
    const double T = cell[13], muB = cell[16], Edec = cell[12], Bn = cell[15];
    coef4[0] = coef4[1] = coef4[2] = 0.0;
    coef4[3] = 1.0;
    if (c->neos_kind == 1) {
        orc_ce_neos(c, Edec, Bn, coef4);
    } else if (c->include_bulk) {
        if (c->bulk_kind == 11) {
            orc_bulk14(c, T, muB, coef4);
        } else if (c->bulk_kind == 1) {
            orc_bulk_rta(T, coef4);
        }
    }
    if (c->include_diff) coef4[3] = orc_qmu_coeff(c, T, muB);
}

void orc_cell_coeffs(const orc_cfg* c, const float* lrf28, int64_t n, double* coef4) {
    for (int64_t l = 0; l < n; l++) orc_cell_coeff_one(c, lrf28 + 28 * l, coef4 + 4 * l);
}

/* ------------------------------------------------------------------------ */
/* FSSW::calculate_dN_analytic, src/FSSW.cpp:719-848 */
static void orc_dN_analytic(const orc_cfg* c, const orc_species* p, double mu, double Temperature,
                            double* res) {
    double N_eq = 0.0, b1 = 0.0, b2 = 0.0, b3 = 0.0, q1 = 0.0, q2 = 0.0;
    const int sign = p->sign;
    const double mass = p->mass;
    const double beta = 1. / Temperature;
    const double lambda = exp(beta * mu);
    const int truncate_order = (mass < 0.7 && Temperature > 0.05) ? 10 : 1;
    for (int n = 1; n <= truncate_order; n++) {
        const double arg = n * mass * beta;
        const double theta = pow(-sign, n - 1);
        const double fugacity = pow(lambda, n);
        const double K_2 = orc_sf_K(c, 2, arg);
        N_eq += theta / n * fugacity * K_2;
        if (c->include_bulk) {
            const double K_1 = orc_sf_K(c, 1, arg);
            if (c->bulk_kind == 1 || c->bulk_kind == 21) {
                b1 += theta * fugacity * (mass * beta * K_1 + 3 * K_2 / n);
                b2 += theta * fugacity * K_1;
            } else if (c->bulk_kind == 11 || c->bulk_kind == 20) {
                const double K_3 = orc_sf_K(c, 3, arg);
                b1 += theta * fugacity * K_2;
                b2 += theta * fugacity * (mass * beta * K_1 + 3 * K_2 / n);
                b3 += theta * fugacity * (mass * beta * K_2 + 3 * K_3 / n);
            }
        }
        if (c->include_diff) {
            q1 += theta / n * fugacity * K_2;
            double En[ORC_N_EXPINT];
            orc_sf_En(c, arg, En);
            const double mbeta = mass * beta;
            const double I11 = exp(-arg) / arg * (2. / (arg * arg) + 2. / arg - 1. / 2.);
            const double I12 = 3. / 8. * En[0];
            double I1n = I11 + I12;
            double dfact = 1., fact = 2., pow2 = 4.;
            for (int k = 3; k <= 10; k++) {
                dfact *= (2 * k - 5);
                fact *= k;
                pow2 *= 2;
                I1n += 3. * dfact / pow2 / fact * En[k - 2];
            }
            I1n = -(mbeta * mbeta * mbeta) * I1n;
            q2 += n * theta * fugacity * I1n;
        }
    }
    N_eq = mass * mass * Temperature * N_eq;
    if (c->include_bulk) {
        if (c->bulk_kind == 1 || c->bulk_kind == 21) {
            b1 = mass * mass / beta * b1;
            b2 = mass * mass * mass / 3. * b2;
            b3 = 0.0;
        } else if (c->bulk_kind == 11 || c->bulk_kind == 20) {
            b1 = mass * mass / beta * b1;
            b2 = mass * mass / (beta * beta) * b2;
            b3 = mass * mass * mass / (beta * beta) * b3;
        }
    } else {
        b1 = b2 = b3 = 0.0;
    }
    if (c->include_diff) {
        q1 = mass * mass / (beta * beta) * q1;
        q2 = 1. / (3. * beta * beta * beta) * q2;
    }
    res[0] = N_eq; res[1] = b1; res[2] = b2; res[3] = b3; res[4] = q1; res[5] = q2;
}

/* FSSW::calculate_dN_dxtdy_for_one_particle_species, src/FSSW.cpp:565-715,
 * for every species (rows of `yields`, mass order) and every cell. */
int orc_yields(const orc_cfg* c, const orc_species* sp, int32_t n_sp, const float* lrf28,
               const int32_t* keep, int64_t n, double* yields) {
    const double unit_factor = 1.0 / pow(ORC_HBARC, 3);
    int status = 0;
    for (int64_t l = 0; l < n; l++) {
        const float* s = lrf28 + 28 * l;
        const double temp = s[13];
        double coef[4];
        orc_cell_coeff_one(c, s, coef);
        const double dsigma_dot_u = s[4];
        double bulkPi = 0.0;
        if (c->include_bulk) {
            if (c->bulk_kind == 21 || c->bulk_kind == 20 || c->bulk_kind == 11 || c->bulk_kind == 0) {
                bulkPi = s[19];
            } else {
                bulkPi = s[19] / ORC_HBARC;
            }
        }
        double dsigma_dot_q = 0.0, kappa = 1.0, prefactor_qmu = 0.0;
        if (c->include_diff) {
            dsigma_dot_q = (s[25] * s[5] + s[26] * s[6] + s[27] * s[7]);
            kappa = coef[3];
            prefactor_qmu = (double)s[15] / ((double)s[12] + (double)s[14]);
        }
        for (int32_t k = 0; k < n_sp; k++) {
            const orc_species* p = sp + k;
            double* out = yields + (int64_t)k * n + l;
            if (keep && !keep[l]) {
                *out = 0.0;
                continue;
            }
            const double mass = p->mass;
            const double mu = p->baryon * s[16] + p->strange * s[17] + p->charge * s[18];
            const double prefactor = p->gspin / (2. * 3.14159265358979323846 * 3.14159265358979323846);
            double r[6];
            orc_dN_analytic(c, p, mu, temp, r);
            if (isnan(r[0])) status = -1;
            const double N_eq = unit_factor * prefactor * dsigma_dot_u * r[0];
            double dNb = 0.0;
            if (c->include_bulk) {
                if (c->bulk_kind == 1 || c->bulk_kind == 21) {
                    dNb = (unit_factor * prefactor * dsigma_dot_u * (-bulkPi * coef[0])
                           * (-coef[1] * r[1] + r[2]));
                } else if (c->bulk_kind == 11) {
                    dNb = (unit_factor * prefactor * dsigma_dot_u * bulkPi
                           * (r[1] * mass * mass * coef[0] + r[2] * p->baryon * coef[1]
                              + r[3] * coef[2]));
                }
            }
            double dNq = 0.0;
            if (c->include_diff) {
                dNq = (unit_factor * prefactor * dsigma_dot_q / kappa
                       * (-prefactor_qmu * r[4] - p->baryon * r[5]));
            }
            const double total = N_eq + dNb + dNq;
            *out = total > 0. ? total : 0.;
        }
    }
    return status;
}

/* Cell CDF of the GPU sampler: RandomVariable1DArray
 * (src/RandomVariable1DArray.cpp:25-74) on fixed-point yields.  Each FP32 yield
 * y of species k becomes q = floor(y * 2^E_k), where E_k = 188 - e_max - L:
 *   - e_max is the biased exponent of the species' largest yield;
 *   - L = ceil(log2 n).
 * So every q < 2^(62-L) and the row sum Q_k < 2^62.  Row k holds the
 * exclusive prefix sums C[0..n] (C[n] = Q_k).  qtot[k] = Q_k and
 * totals[k] = Q_k * 2^-E_k.  Integer sums are exact, so the GPU's tiled scan
 * gives the same bits. */
static int orc_log2_cells(int64_t n) {
    int L = 0;
    while (L < 62 && ((int64_t)1 << L) < n) ++L;
    return L;
}

static uint64_t orc_quantize(uint32_t b, int base) {
    int e = (int)((b >> 23) & 0xFFu);
    uint32_t m = b & 0x7FFFFFu;
    if (e) m |= 0x800000u; else e = 1;
    const int sh = e + base;
    if (sh >= 0) return (uint64_t)m << sh;
    if (sh <= -24) return 0;
    return (uint64_t)(m >> (-sh));
}

void orc_cdf(const float* yields_f32, int32_t n_sp, int64_t n, uint64_t* cdf, uint64_t* qtot,
             double* totals) {
    const int L = orc_log2_cells(n);
    for (int32_t k = 0; k < n_sp; k++) {
        const float* y = yields_f32 + (int64_t)k * n;
        uint32_t ymax = 0;
        for (int64_t l = 0; l < n; l++) {
            float v = y[l];
            if (!(v > 0.0f)) v = 0.0f;            /* negative, -0 and NaN -> +0 */
            if (v > 3.40282347e38f) v = 3.40282347e38f;
            uint32_t b;
            memcpy(&b, &v, 4);
            if (b > ymax) ymax = b;
        }
        int ex = (int)((ymax >> 23) & 0xFFu);
        if (ex == 0) ex = 1;
        const int base = 38 - L - ex;
        uint64_t* row = cdf + (int64_t)k * (n + 1);
        uint64_t sum = 0;
        for (int64_t l = 0; l < n; l++) {
            float v = y[l];
            if (!(v > 0.0f)) v = 0.0f;
            if (v > 3.40282347e38f) v = 3.40282347e38f;
            uint32_t b;
            memcpy(&b, &v, 4);
            row[l] = sum;
            sum += orc_quantize(b, base);
        }
        row[n] = sum;
        qtot[k] = sum;
        totals[k] = sum ? ldexp((double)sum, -(150 + base)) : 0.0;
    }
}

/* ------------------------------------------------------------------------ */
/* Part 2a: counts per (event, species), FSSW::determine_number_to_sample
 * (src/FSSW.cpp:250-309) restated on the Philox stream
 * counter = {iteration, 0, global event, species | TAG_COUNT << 16}. */

typedef struct {
    uint32_t key[2];
    uint32_t ctr[4];
} orc_block_stream;

static void orc_block(orc_block_stream* s, uint32_t iter, uint32_t w[4]) {
    uint32_t ctr[4] = {iter, s->ctr[1], s->ctr[2], s->ctr[3]};
    orc_philox4x32_10(ctr, s->key, w);
}

/* log(k!): lgamma(k + 1) for k < 256, else the Stirling series of
 * lgamma(n), n = k + 1, to the n^-5 term (truncation below 1e-20 relative). */
static double orc_logfact(double kd) {
    static double table[256];
    static int ready = 0;
    if (!ready) {
        for (int i = 0; i < 256; i++) table[i] = lgamma(i + 1.0);
        ready = 1;
    }
    if (kd < 256.0) return table[(int)kd];
    const double n = kd + 1.0;
    const double r = 1.0 / n, r2 = r * r;
    return (n - 0.5) * log(n) - n + 0.91893853320467274178 +
           r * (1.0 / 12.0 - r2 * (1.0 / 360.0 - r2 * (1.0 / 1260.0)));
}

static int64_t orc_poisson(orc_block_stream* s, uint32_t iter0, double mu) {
    uint32_t w[4];
    if (mu < 12.0) {
        orc_block(s, iter0, w);
        const double u = orc_u53(w[0], w[1]);
        double p = exp(-mu);
        double cdf = p;
        int64_t k = 0;
        while (u > cdf && k < 1000) {
            k++;
            p *= mu / (double)k;
            cdf += p;
        }
        return k;
    }
    const double smu = sqrt(mu);
    const double b = 0.931 + 2.53 * smu;
    const double a = -0.059 + 0.02483 * b;
    const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4);
    const double vr = 0.9277 - 3.6224 / (b - 2.0);
    const double log_mu = log(mu);
    for (uint32_t it = 0; it < 10000; it++) {
        orc_block(s, iter0 + it, w);
        const double U = orc_u53(w[0], w[1]) - 0.5;
        const double V = orc_u53(w[2], w[3]);
        const double us = 0.5 - fabs(U);
        const double kd = floor((2.0 * a / us + b) * U + mu + 0.43);
        if (us >= 0.07 && V <= vr) return (int64_t)kd;
        if (kd < 0.0 || (us < 0.013 && V > us)) continue;
        if (log(V) + log(inv_alpha) - log(a / (us * us) + b) <= -mu + kd * log_mu - orc_logfact(kd))
            return (int64_t)kd;
    }
    return -1;
}

/* Gamma(shape, 1) by Marsaglia & Tsang with Box-Muller normals; blocks
 * iter0, iter0+1, ... */
static double orc_gamma(orc_block_stream* s, uint32_t iter0, double shape) {
    uint32_t w[4];
    double boost = 1.0;
    if (shape < 1.0) {
        orc_block(s, iter0, w);
        boost = pow(orc_u01_pos(w[0]), 1.0 / shape);
        shape += 1.0;
        iter0 += 1;
    }
    const double d = shape - 1.0 / 3.0;
    const double cc = 1.0 / sqrt(9.0 * d);
    for (uint32_t it = 0; it < 10000; it++) {
        orc_block(s, iter0 + it, w);
        const double r = sqrt(-2.0 * log(orc_u01_pos(w[0])));
        const double x = r * cos(2.0 * 3.14159265358979323846 * orc_u01(w[1]));
        double v = 1.0 + cc * x;
        if (v <= 0.0) continue;
        v = v * v * v;
        const double u = orc_u53(w[2], w[3]);
        if (u < 1.0 - 0.0331 * x * x * x * x) return boost * d * v;
        if (log(u) < 0.5 * x * x + d * (1.0 - v + log(v))) return boost * d * v;
    }
    return -1.0;
}

int orc_counts(const orc_cfg* c, const orc_species* sp, int32_t n_sp, const double* totals,
               int32_t* counts) {
    const double ymult = (c->hydro_mode != 2) ? (c->y_rb - c->y_lb) : 1.0;
    for (int64_t e = 0; e < c->n_events; e++) {
        const uint64_t eg = (uint64_t)(c->event_offset + e);
        for (int32_t k = 0; k < n_sp; k++) {
            orc_block_stream s;
            s.key[0] = (uint32_t)c->seed;
            s.key[1] = (uint32_t)(c->seed >> 32);
            s.ctr[0] = 0;
            s.ctr[1] = 0;
            s.ctr[2] = (uint32_t)eg;
            s.ctr[3] = (uint32_t)k | ((uint32_t)ORC_TAG_COUNT << 16);
            const double dN = totals[k] * ymult;
            int64_t n = 0;
            /* local_charge_conservation: negative species are not drawn; a
             * positive species' segment holds two records per draw */
            if (c->lcc && sp[k].charge < 0) {
                counts[e * n_sp + k] = 0;
                continue;
            }
            const int mult = (c->lcc && sp[k].charge > 0) ? 2 : 1;
            if (dN < 0) return -2;
            const int64_t dN_int = (int64_t)dN;
            const double frac = dN - (double)dN_int;
            const double para1 = c->sampling_para1;
            switch (c->sampling_model) {
                case 1: {
                    uint32_t w[4];
                    orc_block(&s, 0, w);
                    n = dN_int + (orc_u53(w[0], w[1]) < frac ? 1 : 0);
                    break;
                }
                case 10: {
                    const double kk = para1 * frac;
                    const double p = 1.0 / (1.0 + para1);
                    if (kk < 1e-15) {
                        n = dN_int;
                    } else {
                        const double g = orc_gamma(&s, 0, kk);
                        n = dN_int + orc_poisson(&s, 1u << 20, g * (1.0 - p) / p);
                    }
                    break;
                }
                case 20: {
                    const double kk = para1 * dN;
                    const double p = 1.0 / (1.0 + para1);
                    if (kk < 1e-15) {
                        n = dN_int;
                    } else {
                        const double g = orc_gamma(&s, 0, kk);
                        n = orc_poisson(&s, 1u << 20, g * (1.0 - p) / p);
                    }
                    break;
                }
                case 30:
                    n = (dN < 1e-15) ? 0 : orc_poisson(&s, 0, dN);
                    break;
                default:
                    return -3;
            }
            if (n < 0) return -4;
            counts[e * n_sp + k] = (int32_t)(n * mult);
        }
    }
    return 0;
}
