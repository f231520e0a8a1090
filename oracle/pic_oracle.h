/*
 * pic_oracle.h -- C interface of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a CPU restatement of the
 * reference cycle (AntonioTejero/cupic, src/mesh.cu, src/particles.cu,
 * src/cc.cu, src/init.cu) that tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py check and time against.  Nothing in the
 * product path (cupic_gb300/) links or calls it.
 *
 * Two precisions share one code path:
 *   fp64=1  all-FP64 "precision oracle": double particles, double charge
 *           sums, double Jacobi -- the reference's arithmetic with the
 *           defects listed in pic_oracle.cpp fixed.
 *   fp64=0  FP32 "parity oracle": the exact operation sequence of the GPU
 *           kernels (float particles, int64 fixed-point charge, float
 *           Jacobi, explicit fma), so GPU results can be compared bit for bit.
 */
#ifndef CUPIC_PIC_ORACLE_H
#define CUPIC_PIC_ORACLE_H

#include <stdint.h>
#include "../include/cupic_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

void *ora_create(const cupic_params *p, int fp64);
void ora_destroy(void *h);
void ora_set_threads(int n);

int ora_params_from_input_data(const char *path, cupic_params *p);
int ora_params_default(cupic_params *p);

int ora_init_plasma(void *h);
int ora_load(void *h, int species, const double *xyvv, int64_t n);
int ora_set_time(void *h, int64_t step, double t, double tin_e, double tin_i);
int ora_get_time(void *h, int64_t *step, double *t, double *tin_e, double *tin_i);

int ora_deposit(void *h);
int ora_solve(void *h, double tol, int32_t min_sweeps, int32_t max_sweeps, int32_t check_every,
              int32_t *sweeps, double *residual);
int ora_field(void *h);
/* mode 0: full push + wrap + binning; mode 1: leapfrog start (v -= dt/2 qE/m) */
int ora_push(void *h, int mode);
int ora_inject(void *h, double t);
int ora_step(void *h, int32_t nsteps);

int ora_get_counts(void *h, int64_t *ne, int64_t *ni);
int ora_get_particles(void *h, int species, double *xyvv);
int ora_get_row_counts(void *h, int species, int32_t *counts);
/* E at every particle of a species (the push's CIC gather), in row order */
int ora_gather(void *h, int species, double *ex, double *ey);
int ora_get_phi(void *h, double *phi);
int ora_set_phi(void *h, const double *phi);
int ora_get_field(void *h, double *ex, double *ey);
int ora_get_rho(void *h, int which, double *rho);
int ora_get_rho_fixed(void *h, int64_t *acc);
int ora_get_stats(void *h, cupic_step_stats *st);
uint32_t ora_get_flags(void *h);

/* primitives, for known-answer tests */
void ora_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double ora_log(double x);
void ora_sincos2pi(double u, double *s, double *c);

#ifdef __cplusplus
}
#endif

#endif
