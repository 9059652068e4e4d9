// Test infrastructure only (oracle side): GSL-compatible special functions and
// random variates, so that the unmodified reference sources (which call GSL at
// FSSW.cpp:169-172, 282, 291, 297, 1626-1639, 1655, 1675, 1695, 1715-1717 and
// emissionfunction.cpp) compile and run here without GSL installed.
//
// Every routine is written from the mathematics, not from GSL:
//  * K_nu(x) = int_0^inf exp(-x cosh t) cosh(nu t) dt, evaluated with the
//    trapezoidal rule, which converges geometrically for this entire,
//    double-exponentially decaying integrand (Trefethen & Weideman, SIAM Rev.
//    56 (2014) 385).  The step is h = min(0.02, 0.5/sqrt(x)); the discretisation
//    error then stays below exp(-2 pi^2/(h^2 x)) < 1e-30.
//  * E_n(x): power series (Abramowitz & Stegun 5.1.12) for x <= 1 and the
//    continued fraction (A&S 5.1.22) evaluated with the modified Lentz method
//    for x > 1.
//  * Lambert W0: Halley iteration.
//  * Poisson: sequential inversion for mu < 12, Hormann's PTRS transformed
//    rejection (Insurance: Math. Econ. 12 (1993) 39) otherwise.
//  * Gamma: Marsaglia & Tsang (ACM TOMS 26 (2000) 363); negative binomial as a
//    Poisson-gamma mixture.
// The uniform generator behind gsl_rng is std::mt19937 (32-bit output / 2^32).
#include <cmath>
#include <cstdlib>
#include <random>
#include "gsl/gsl_sf_bessel.h"
#include "gsl/gsl_sf_expint.h"
#include "gsl/gsl_sf_lambert.h"
#include "gsl/gsl_rng.h"
#include "gsl/gsl_randist.h"

namespace {

double bessel_k_scaled(double nu, double x) {
    // returns exp(x) * K_nu(x)
    if (!(x > 0.0)) return HUGE_VAL;
    double h = 0.5 / std::sqrt(x);
    if (h > 0.02) h = 0.02;
    double sum = 0.5;  // t = 0 term: exp(0)*cosh(0), half weight
    for (int k = 1; k < 200000; k++) {
        const double t = k * h;
        const double e = -x * (std::cosh(t) - 1.0) + nu * t;
        const double term = std::exp(e) * 0.5 * (1.0 + std::exp(-2.0 * nu * t));
        sum += term;
        if (e < -60.0 && term < 1e-30 * sum) break;
    }
    return sum * h;
}

double expint_series(int n, double x) {
    // A&S 5.1.12, valid for all x > 0 but used for x <= 1
    const double euler = 0.57721566490153286061;
    double psi = -euler;
    for (int k = 1; k <= n - 1; k++) psi += 1.0 / k;
    double result;
    if (n - 1 != 0) {
        result = 1.0 / (n - 1);
    } else {
        result = -std::log(x) - euler;
    }
    double fact = 1.0;  // (-x)^m / m!
    for (int m = 1; m < 1000; m++) {
        fact *= -x / m;
        double del;
        if (m != n - 1) {
            del = -fact / (m - n + 1);
        } else {
            del = fact * (-std::log(x) + psi);
        }
        result += del;
        if (std::fabs(del) < std::fabs(result) * 1e-17) break;
    }
    return result;
}

double expint_cfrac(int n, double x) {
    // A&S 5.1.22 with the modified Lentz algorithm
    const double tiny = 1e-300;
    double b = x + n;
    double c = 1.0 / tiny;
    double d = 1.0 / b;
    double h = d;
    for (int i = 1; i < 10000; i++) {
        const double an = -static_cast<double>(i) * (n - 1 + i);
        b += 2.0;
        d = 1.0 / (an * d + b);
        c = b + an / c;
        const double del = c * d;
        h *= del;
        if (std::fabs(del - 1.0) < 1e-17) break;
    }
    return h * std::exp(-x);
}

}  // namespace

extern "C" {

double gsl_sf_bessel_K0(double x) { return bessel_k_scaled(0.0, x) * std::exp(-x); }
double gsl_sf_bessel_K1(double x) { return bessel_k_scaled(1.0, x) * std::exp(-x); }
double gsl_sf_bessel_Kn(int n, double x) {
    return bessel_k_scaled(static_cast<double>(std::abs(n)), x) * std::exp(-x);
}

double gsl_sf_expint_En(int n, double x) {
    if (n == 0) return std::exp(-x) / x;
    if (x <= 0.0) return (n > 1) ? 1.0 / (n - 1) : HUGE_VAL;
    if (x > 1.0) return expint_cfrac(n, x);
    return expint_series(n, x);
}
double gsl_sf_expint_E1(double x) { return gsl_sf_expint_En(1, x); }
double gsl_sf_expint_E2(double x) { return gsl_sf_expint_En(2, x); }

double gsl_sf_lambert_W0(double x) {
    if (x == 0.0) return 0.0;
    const double branch = -1.0 / std::exp(1.0);
    if (x <= branch) return -1.0;
    double w = (x < 1.0) ? x * (1.0 - x) : std::log(1.0 + x);
    if (x < 0.0) w = -1.0 + std::sqrt(2.0 * (1.0 + std::exp(1.0) * x));
    for (int it = 0; it < 100; it++) {
        const double ew = std::exp(w);
        const double f = w * ew - x;
        const double wp1 = w + 1.0;
        const double denom = ew * wp1 - (w + 2.0) * f / (2.0 * wp1);
        const double dw = f / denom;
        w -= dw;
        if (std::fabs(dw) <= 1e-16 * (1.0 + std::fabs(w))) break;
    }
    return w;
}

struct gsl_rng {
    std::mt19937 gen;
};

static const gsl_rng_type mt_type = {"mt19937"};
const gsl_rng_type* gsl_rng_mt19937 = &mt_type;
const gsl_rng_type* gsl_rng_default = &mt_type;

const gsl_rng_type* gsl_rng_env_setup(void) { return gsl_rng_default; }

gsl_rng* gsl_rng_alloc(const gsl_rng_type*) {
    gsl_rng* r = new gsl_rng;
    r->gen.seed(4357u);
    return r;
}

void gsl_rng_set(const gsl_rng* r, unsigned long seed) {
    const_cast<gsl_rng*>(r)->gen.seed(static_cast<std::mt19937::result_type>(seed));
}

void gsl_rng_free(gsl_rng* r) { delete r; }

double gsl_rng_uniform(const gsl_rng* r) {
    return const_cast<gsl_rng*>(r)->gen() / 4294967296.0;
}

double gsl_rng_uniform_pos(const gsl_rng* r) {
    double u;
    do { u = gsl_rng_uniform(r); } while (u == 0.0);
    return u;
}

unsigned int gsl_ran_poisson(const gsl_rng* r, double mu) {
    if (!(mu > 0.0)) return 0u;
    if (mu < 12.0) {
        const double u = gsl_rng_uniform(r);
        double p = std::exp(-mu);
        double cdf = p;
        unsigned int k = 0;
        while (u > cdf && k < 100000u) {
            k++;
            p *= mu / k;
            cdf += p;
            if (p < 1e-300) break;
        }
        return k;
    }
    const double smu = std::sqrt(mu);
    const double b = 0.931 + 2.53 * smu;
    const double a = -0.059 + 0.02483 * b;
    const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4);
    const double vr = 0.9277 - 3.6224 / (b - 2.0);
    const double log_mu = std::log(mu);
    for (;;) {
        const double U = gsl_rng_uniform(r) - 0.5;
        const double V = gsl_rng_uniform(r);
        const double us = 0.5 - std::fabs(U);
        const double kd = std::floor((2.0 * a / us + b) * U + mu + 0.43);
        if (us >= 0.07 && V <= vr) return static_cast<unsigned int>(kd);
        if (kd < 0.0 || (us < 0.013 && V > us)) continue;
        if (std::log(V) + std::log(inv_alpha) - std::log(a / (us * us) + b)
            <= -mu + kd * log_mu - std::lgamma(kd + 1.0)) {
            return static_cast<unsigned int>(kd);
        }
    }
}

double gsl_ran_gamma(const gsl_rng* r, double a, double b) {
    if (a < 1.0) {
        const double u = gsl_rng_uniform_pos(r);
        return gsl_ran_gamma(r, 1.0 + a, b) * std::pow(u, 1.0 / a);
    }
    const double d = a - 1.0 / 3.0;
    const double c = 1.0 / std::sqrt(9.0 * d);
    std::normal_distribution<double> normal(0.0, 1.0);
    for (;;) {
        double x, v;
        do {
            x = normal(const_cast<gsl_rng*>(r)->gen);
            v = 1.0 + c * x;
        } while (v <= 0.0);
        v = v * v * v;
        const double u = gsl_rng_uniform_pos(r);
        if (u < 1.0 - 0.0331 * x * x * x * x) return b * d * v;
        if (std::log(u) < 0.5 * x * x + d * (1.0 - v + std::log(v))) return b * d * v;
    }
}

unsigned int gsl_ran_negative_binomial(const gsl_rng* r, double p, double n) {
    const double x = gsl_ran_gamma(r, n, 1.0);
    return gsl_ran_poisson(r, x * (1.0 - p) / p);
}

}  // extern "C"
