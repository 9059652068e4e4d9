/* Test infrastructure only: minimal GSL-compatible declarations so that the
 * unmodified reference sources compile here for use as an oracle.
 * Implementations live in oracle/gsl_compat/gsl_compat.cpp (written from the
 * integral representation of K_nu, not from GSL). */
#ifndef ISS_ORACLE_GSL_SF_BESSEL_H
#define ISS_ORACLE_GSL_SF_BESSEL_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_bessel_K0(double x);
double gsl_sf_bessel_K1(double x);
double gsl_sf_bessel_Kn(int n, double x);
#ifdef __cplusplus
}
#endif
#endif
