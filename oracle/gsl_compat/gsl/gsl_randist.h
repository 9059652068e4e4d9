/* Test infrastructure only: Poisson and negative-binomial variates with the
 * GSL calling convention (see oracle/gsl_compat/gsl_compat.cpp). */
#ifndef ISS_ORACLE_GSL_RANDIST_H
#define ISS_ORACLE_GSL_RANDIST_H
#include "gsl_rng.h"
#ifdef __cplusplus
extern "C" {
#endif
unsigned int gsl_ran_poisson(const gsl_rng* r, double mu);
double gsl_ran_gamma(const gsl_rng* r, double a, double b);
unsigned int gsl_ran_negative_binomial(const gsl_rng* r, double p, double n);
#ifdef __cplusplus
}
#endif
#endif
