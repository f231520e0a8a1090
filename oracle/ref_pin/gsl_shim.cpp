// Project-written stand-ins for the six GSL symbols the reference uses
// (gslrand.h).  TEST INFRASTRUCTURE ONLY; the pin harness never draws from
// them.  Generator: splitmix64 (Steele, Lea, Flood 2014); normal by
// Box-Muller; Rayleigh by inverting its CDF, sigma*sqrt(-2 ln u).
#include <cmath>
#include <cstdlib>
#include "gsl/gsl_randist.h"
static const gsl_rng_type kType = {"splitmix64"};
const gsl_rng_type *gsl_rng_default = &kType;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *) {
  gsl_rng *r = (gsl_rng *)std::malloc(sizeof(gsl_rng));
  r->state = 0x853c49e6748fea9bULL;
  return r;
}
const gsl_rng_type *gsl_rng_env_setup(void) { return gsl_rng_default; }
static unsigned long long next(const gsl_rng *r) {
  gsl_rng *m = const_cast<gsl_rng *>(r);
  unsigned long long z = (m->state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
double gsl_rng_uniform_pos(const gsl_rng *r) { return ((double)(next(r) >> 11) + 0.5) * 0x1p-53; }
double gsl_ran_gaussian(const gsl_rng *r, double sigma) {
  const double u = gsl_rng_uniform_pos(r), v = gsl_rng_uniform_pos(r);
  return sigma * std::sqrt(-2.0 * std::log(u)) * std::cos(6.283185307179586 * v);
}
double gsl_ran_rayleigh(const gsl_rng *r, double sigma) {
  return sigma * std::sqrt(-2.0 * std::log(gsl_rng_uniform_pos(r)));
}
