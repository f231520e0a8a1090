/* Minimal GSL distribution API (see gsl_rng.h); TEST INFRASTRUCTURE ONLY. */
#ifndef CUPIC_PIN_GSL_RANDIST_H
#define CUPIC_PIN_GSL_RANDIST_H
#include "gsl_rng.h"
#ifdef __cplusplus
extern "C" {
#endif
double gsl_ran_gaussian(const gsl_rng *r, double sigma);
double gsl_ran_rayleigh(const gsl_rng *r, double sigma);
#ifdef __cplusplus
}
#endif
#endif
