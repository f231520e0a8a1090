/*
 * cupic_ref.h -- the reference's C++ host surface, implemented over the
 * C-ABI of cupic_gpu.h (library libcupic_ref.so).
 *
 * The functions keep the reference's names, signatures and call order, so
 * its unchanged src/main.cu links against libcupic_ref.so + libcupic_gpu.so
 * in place of its own init/cc/mesh/particles/diagnostic/cuda objects:
 *   init.h:32-63       init_dev, init_sim, the init_* parameter getters
 *   mesh.h:27-29       charge_deposition, poisson_solver, field_solver
 *   particles.h:28     particle_mover
 *   cc.h:29            cc
 *   diagnostic.h:27-31 number_of_particles, particles_snapshot,
 *                      mesh_snapshot, save_bm, save_bins
 *   cuda.h:28          cuda_reset
 * The state lives in one process-wide cupic context created by init_sim.
 * The pointers init_sim hands out (d_rho, d_e, d_e_bm, ...) are opaque
 * handles that name an array of that context; they are not device pointers
 * and must not be dereferenced.  As in the reference, errors print a
 * message and exit(1).
 */
#ifndef CUPIC_REF_H
#define CUPIC_REF_H

#include <string>

struct particle {  // stdh.h:30-36
  double x;
  double y;
  double vx;
  double vy;
};

void init_dev(void);
void init_sim(double **d_rho, double **d_phi, double **d_Ex, double **d_Ey, particle **d_e,
              particle **d_i, int **d_e_bm, int **d_i_bm, double *t);
double init_qi(void);
double init_qe(void);
double init_mi(void);
double init_me(void);
double init_kti(void);
double init_kte(void);
double init_phi_p(void);
double init_n(void);
double init_Lx(void);
double init_Ly(void);
double init_ds(void);
double init_dt(void);
double init_dtin_i(void);
double init_dtin_e(void);
double init_epsilon0(void);
int init_ncx(void);
int init_ncy(void);
int init_nnx(void);
int init_nny(void);
int init_n_ini(void);
int init_n_prev(void);
int init_n_save(void);
int init_n_fin(void);

void charge_deposition(double *d_rho, particle *d_e, int *d_e_bm, particle *d_i, int *d_i_bm);
void poisson_solver(double max_error, double *d_rho, double *d_phi);
void field_solver(double *d_phi, double *d_Ex, double *d_Ey);
void particle_mover(particle *d_e, int *d_e_bm, particle *d_i, int *d_i_bm, double *Ex, double *Ey);
void cc(double t, int *d_e_bm, particle **d_e, int *d_i_bm, particle **d_i, double *d_Ex,
        double *d_Ey);

int number_of_particles(int *d_bm);
void particles_snapshot(particle *d_p, int *d_bm, std::string filename, double t);
void mesh_snapshot(double *d_m, std::string filename);
void save_bm(int *d_bm, std::string filename);
void save_bins(int *d_bm, particle *d_p, std::string filename);
void cuda_reset(double **d_rho, double **d_phi, double **d_Ex, double **d_Ey, particle **d_e,
                particle **d_i, int **d_e_bm, int **d_i_bm);

#endif
