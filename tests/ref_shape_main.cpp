// A driver in the shape of the reference's main loop (src/main.cu:26-117),
// written against the reference-named functions of include/cupic_ref.h and
// linked with libcupic_ref.so.  Used by tests/test_gpu_driver.py to show
// that a main of that shape runs unchanged on the GB300 library.
#include <stdio.h>

#include <fstream>
#include <iostream>
#include <string>

#include "cupic_ref.h"

static std::string name(const char *species, int i) {
  char buf[64];
  snprintf(buf, sizeof buf, "../output/particles/%s_t_%d", species, i);
  return buf;
}

int main() {
  const double dt = init_dt();
  const int first = init_n_ini(), prev = init_n_prev(), every = init_n_save(), last = init_n_fin();
  double *rho, *phi, *ex, *ey;
  particle *e, *ions;
  int *e_bm, *i_bm;
  double t;

  init_dev();
  init_sim(&rho, &phi, &ex, &ey, &e, &ions, &e_bm, &i_bm, &t);
  std::cout << "t = " << t << std::endl;
  particles_snapshot(e, e_bm, name("electrons", first), t);
  particles_snapshot(ions, i_bm, name("ions", first), t);
  t += dt;

  for (int step = first + 1; step <= last; ++step, t += dt) {
    charge_deposition(rho, e, e_bm, ions, i_bm);
    poisson_solver(1.0e-4, rho, phi);
    field_solver(phi, ex, ey);
    particle_mover(e, e_bm, ions, i_bm, ex, ey);
    cc(t, e_bm, &e, i_bm, &ions, ex, ey);
    if (step % 10000 == 0) cuda_reset(&rho, &phi, &ex, &ey, &e, &ions, &e_bm, &i_bm);
    if (step >= prev && step % every == 0) {
      particles_snapshot(e, e_bm, name("electrons", step), t);
      particles_snapshot(ions, i_bm, name("ions", step), t);
      mesh_snapshot(rho, "../output/charge_t_" + std::to_string(step - 1));
      mesh_snapshot(phi, "../output/potential_t_" + std::to_string(step - 1));
      save_bm(e_bm, "bm_electrons_t_" + std::to_string(step));
      save_bins(e_bm, e, "bins_electrons_t_" + std::to_string(step));
    }
    std::cout << "t = " << t << std::endl;
  }
  std::cout << "Simulation finished!" << std::endl;
  return 0;
}
