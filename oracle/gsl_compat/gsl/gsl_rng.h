/* Test infrastructure only: the subset of the GSL random-number-generator
 * interface used by the reference (allocation, seeding, uniform draws).
 * The generator behind it is a 32-bit Mersenne twister. */
#ifndef ISS_ORACLE_GSL_RNG_H
#define ISS_ORACLE_GSL_RNG_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct gsl_rng_type { const char* name; } gsl_rng_type;
typedef struct gsl_rng gsl_rng;
extern const gsl_rng_type* gsl_rng_default;
extern const gsl_rng_type* gsl_rng_mt19937;
const gsl_rng_type* gsl_rng_env_setup(void);
gsl_rng* gsl_rng_alloc(const gsl_rng_type* T);
void gsl_rng_set(const gsl_rng* r, unsigned long seed);
void gsl_rng_free(gsl_rng* r);
double gsl_rng_uniform(const gsl_rng* r);
double gsl_rng_uniform_pos(const gsl_rng* r);
#ifdef __cplusplus
}
#endif
#endif
