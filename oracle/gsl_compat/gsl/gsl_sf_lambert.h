/* Test infrastructure only: GSL-compatible declaration of the principal
 * branch of the Lambert W function (needed only to link the reference's
 * legacy sampler; see oracle/gsl_compat/gsl_compat.cpp). */
#ifndef ISS_ORACLE_GSL_SF_LAMBERT_H
#define ISS_ORACLE_GSL_SF_LAMBERT_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_lambert_W0(double x);
#ifdef __cplusplus
}
#endif
#endif
