/* Minimal GSL random-number API, written for this project from the
 * mathematics (not from GSL's sources), so that the reference's sources
 * compile and link here.  TEST INFRASTRUCTURE ONLY: it lets the reference's
 * input_data getters be run to pin the oracle's normalisation. */
#ifndef CUPIC_PIN_GSL_RNG_H
#define CUPIC_PIN_GSL_RNG_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct gsl_rng_type { const char *name; } gsl_rng_type;
typedef struct gsl_rng { unsigned long long state; } gsl_rng;
extern const gsl_rng_type *gsl_rng_default;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *t);
const gsl_rng_type *gsl_rng_env_setup(void);
double gsl_rng_uniform_pos(const gsl_rng *r);
#ifdef __cplusplus
}
#endif
#endif
