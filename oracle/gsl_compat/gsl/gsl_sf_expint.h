/* Test infrastructure only: GSL-compatible declarations of the exponential
 * integrals E_n used by the reference (see oracle/gsl_compat/gsl_compat.cpp). */
#ifndef ISS_ORACLE_GSL_SF_EXPINT_H
#define ISS_ORACLE_GSL_SF_EXPINT_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_expint_E1(double x);
double gsl_sf_expint_E2(double x);
double gsl_sf_expint_En(int n, double x);
#ifdef __cplusplus
}
#endif
#endif
