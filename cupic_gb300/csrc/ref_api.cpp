// ref_api.cpp -- the reference's C++ host functions (include/cupic_ref.h)
// over the C-ABI.  One process-wide context, created by init_sim; the
// reference's device pointers become handles naming that context's arrays.
#include "cupic_ref.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <iostream>
#include <string>

#include "cupic_gpu.h"

namespace {

const char *const kInput = "../input/input_data";  // init.cu:424-447

struct Handles {
  double rho, phi, ex, ey;
  particle e, i;
  int e_bm, i_bm;
};
Handles g_tags;
cupic_ctx *g_ctx = nullptr;

void die(const char *what, int rc) {
  std::cout << "cupic: " << what << ": " << cupic_strerror(rc) << std::endl;
  exit(1);
}

void check(int rc, const char *what) {
  if (rc) die(what, rc);
}

// the parameters, read once like the reference's static getters
const cupic_params &params() {
  static cupic_params p;
  static bool read = false;
  if (!read) {
    check(cupic_params_from_input_data(kInput, &p), kInput);
    read = true;
  }
  return p;
}

cupic_ctx *ctx() {
  if (!g_ctx) die("init_sim has not run", CUPIC_ERR_STATE);
  return g_ctx;
}

int species_of(const particle *p) {
  if (p == &g_tags.e) return 0;
  if (p == &g_tags.i) return 1;
  die("unknown particle array", CUPIC_ERR_ARG);
  return -1;
}

int species_of_bm(const int *bm) {
  if (bm == &g_tags.e_bm) return 0;
  if (bm == &g_tags.i_bm) return 1;
  die("unknown bookmark array", CUPIC_ERR_ARG);
  return -1;
}

double dtin(double m, double kt) {  // init.cu:686-714
  const cupic_params &p = params();
  return sqrt(2.0 * 3.1415926535897932 * m / kt) / (p.n * (p.ds * p.ncx) * p.ds);
}

}  // namespace

void init_dev(void) {}

void init_sim(double **d_rho, double **d_phi, double **d_Ex, double **d_Ey, particle **d_e,
              particle **d_i, int **d_e_bm, int **d_i_bm, double *t) {
  const cupic_params &p = params();
  if (!g_ctx) check(cupic_create(&p, 0, &g_ctx), "create");
  if (p.n_ini == 0) {  // init.cu:70-83
    *t = 0.;
    check(cupic_init_plasma(g_ctx), "init_sim");
    int64_t ne = 0, ni = 0;
    check(cupic_get_counts(g_ctx, &ne, &ni), "init_sim");
    std::cout << "Simulation initialized with " << ne * 2 << " particles." << std::endl << std::endl;
  } else if (p.n_ini > 0) {  // init.cu:84-93
    *t = p.n_ini * p.dt;
    check(cupic_load_particles_file(g_ctx, 1, "./ions.dat"), "./ions.dat");
    check(cupic_load_particles_file(g_ctx, 0, "./electrons.dat"), "./electrons.dat");
    check(cupic_init_mesh(g_ctx), "init_sim");
    std::cout << "Simulation state loaded from time t = " << *t << std::endl;
  } else {
    std::cout << "Wrong input parameter (n_ini<0)" << std::endl;
    std::cout << "Stoppin simulation" << std::endl;
    exit(1);
  }
  *d_rho = &g_tags.rho;
  *d_phi = &g_tags.phi;
  *d_Ex = &g_tags.ex;
  *d_Ey = &g_tags.ey;
  *d_e = &g_tags.e;
  *d_i = &g_tags.i;
  *d_e_bm = &g_tags.e_bm;
  *d_i_bm = &g_tags.i_bm;
}

double init_qi(void) { return params().qi; }
double init_qe(void) { return params().qe; }
double init_mi(void) { return params().mi; }
double init_me(void) { return params().me; }
double init_kti(void) { return params().kti; }
double init_kte(void) { return params().kte; }
double init_phi_p(void) { return params().phi_p; }
double init_n(void) { return params().n; }
double init_Lx(void) { return params().ds * params().ncx; }
double init_Ly(void) { return params().ds * params().ncy; }
double init_ds(void) { return params().ds; }
double init_dt(void) { return params().dt; }
double init_dtin_i(void) { return dtin(params().mi, params().kti); }
double init_dtin_e(void) { return dtin(params().me, params().kte); }
double init_epsilon0(void) { return params().eps0; }
int init_ncx(void) { return params().ncx; }
int init_ncy(void) { return params().ncy; }
int init_nnx(void) { return params().ncx + 1; }
int init_nny(void) { return params().ncy + 1; }
int init_n_ini(void) { return params().n_ini; }
int init_n_prev(void) { return params().n_prev; }
int init_n_save(void) { return params().n_save; }
int init_n_fin(void) { return params().n_fin; }

void charge_deposition(double *, particle *, int *, particle *, int *) {
  check(cupic_charge_deposition(ctx()), "charge_deposition");
}

// mesh.cu:55-120: at least max(nnx, nny)+1 sweeps, then until max |dphi| < max_error
void poisson_solver(double max_error, double *, double *) {
  const cupic_params &p = params();
  check(cupic_poisson_solver(ctx(), max_error, p.min_sweeps, p.max_sweeps, 1), "poisson_solver");
}

void field_solver(double *, double *, double *) {
  check(cupic_field_solver(ctx()), "field_solver");
}

void particle_mover(particle *, int *, particle *, int *, double *, double *) {
  check(cupic_particle_mover(ctx()), "particle_mover");
}

void cc(double t, int *, particle **, int *, particle **, double *, double *) {
  check(cupic_cc(ctx(), t), "cc");
}

int number_of_particles(int *d_bm) {
  int64_t ne = 0, ni = 0;
  check(cupic_get_counts(ctx(), &ne, &ni), "number_of_particles");
  return (int)(species_of_bm(d_bm) == 0 ? ne : ni);
}

void particles_snapshot(particle *d_p, int *, std::string filename, double) {
  filename.append(".dat");  // diagnostic.cu:74
  check(cupic_particles_snapshot(ctx(), species_of(d_p), filename.c_str()), filename.c_str());
}

void mesh_snapshot(double *d_m, std::string filename) {
  int what;
  if (d_m == &g_tags.rho)
    what = 1;  // the charge the last solve used: the reference's d_rho after a step
  else if (d_m == &g_tags.phi)
    what = 2;
  else if (d_m == &g_tags.ex)
    what = 3;
  else if (d_m == &g_tags.ey)
    what = 4;
  else
    die("unknown mesh array", CUPIC_ERR_ARG);
  filename.append(".dat");  // diagnostic.cu:115
  check(cupic_mesh_snapshot(ctx(), what, filename.c_str()), filename.c_str());
}

void save_bm(int *d_bm, std::string filename) {
  filename.insert(0, "../output/");  // diagnostic.cu:157-158
  filename.append(".dat");
  check(cupic_save_bm(ctx(), species_of_bm(d_bm), filename.c_str()), filename.c_str());
}

void save_bins(int *, particle *d_p, std::string filename) {
  filename.insert(0, "../output/");  // diagnostic.cu:200-201
  filename.append(".dat");
  check(cupic_save_bins(ctx(), species_of(d_p), filename.c_str()), filename.c_str());
}

// The reference copies everything out, resets the device and copies it back
// to undo fragmentation (cuda.cu:58-164); this storage never fragments.
void cuda_reset(double **, double **, double **, double **, particle **, particle **, int **,
                int **) {}
