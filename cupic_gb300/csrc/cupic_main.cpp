// cupic_main.cpp -- the reference's program (src/main.cu:26-117) on the GB300
// library: it reads the same input_data, writes the same particle files and
// prints the same console lines, and it rewrites n_ini at the end.
//
//   cupic_run [--stages] [input_data [output_dir [restart_dir]]]
//
// The defaults are the reference's paths: ../input/input_data, ../output, and
// "." for the restart files ions.dat / electrons.dat (init.cu:338-341).
// Between two saves the cycle runs as captured CUDA graphs with no host
// synchronisation (cupic_step); --stages instead calls the five stages one
// by one per step, as the reference's loop does (main.cu:59-73).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>

#include "cupic_gpu.h"

namespace {

int fail(const char *what, int rc) {
  fprintf(stderr, "cupic: %s: %s\n", what, cupic_strerror(rc));
  return 1;
}

std::string particle_file(const std::string &dir, const char *species, int i) {
  return dir + "/particles/" + species + "_t_" + std::to_string(i) + ".dat";  // main.cu:53,80
}

int snapshot(cupic_ctx *ctx, const std::string &dir, int i) {
  int rc = cupic_particles_snapshot(ctx, 0, particle_file(dir, "electrons", i).c_str());
  if (!rc) rc = cupic_particles_snapshot(ctx, 1, particle_file(dir, "ions", i).c_str());
  return rc;
}

}  // namespace

int main(int argc, char **argv) {
  bool stages = false;
  const char *pos[3] = {"../input/input_data", "../output", "."};
  int npos = 0;
  for (int a = 1; a < argc; ++a) {
    if (!strcmp(argv[a], "--stages"))
      stages = true;
    else if (npos < 3)
      pos[npos++] = argv[a];
  }
  const std::string input = pos[0], out = pos[1], restart = pos[2];

  cupic_params p;
  int rc = cupic_params_from_input_data(input.c_str(), &p);
  if (rc) return fail(input.c_str(), rc);
  const double dt = p.dt;
  const int n_ini = p.n_ini, n_prev = p.n_prev, n_save = p.n_save, n_fin = p.n_fin;
  if (n_save <= 0) return fail("n_save must be positive", CUPIC_ERR_ARG);

  cupic_ctx *ctx = nullptr;
  rc = cupic_create(&p, 0, &ctx);
  if (rc) return fail("create", rc);

  double t;
  if (n_ini == 0) {  // init.cu:70-83
    t = 0.;
    rc = cupic_init_plasma(ctx);
    if (rc) return fail("init", rc);
    int64_t ne = 0, ni = 0;
    cupic_get_counts(ctx, &ne, &ni);
    printf("Simulation initialized with %lld particles.\n\n", (long long)(2 * ne));
  } else if (n_ini > 0) {  // init.cu:84-93
    t = n_ini * dt;
    rc = cupic_load_particles_file(ctx, 1, (restart + "/ions.dat").c_str());
    if (!rc) rc = cupic_load_particles_file(ctx, 0, (restart + "/electrons.dat").c_str());
    if (!rc) rc = cupic_init_mesh(ctx);
    if (rc) return fail("restart", rc);
    printf("Simulation state loaded from time t = %g\n", t);
  } else {
    printf("Wrong input parameter (n_ini<0)\nStoppin simulation\n");
    return 1;
  }

  printf("t = %g\n", t);
  rc = snapshot(ctx, out, n_ini);
  if (rc) return fail("snapshot", rc);
  t += dt;

  for (int i = n_ini + 1; i <= n_fin;) {
    // run up to the next step that saves (or the last one)
    int last = n_fin;
    for (int k = i; k <= n_fin; ++k)
      if (k >= n_prev && k % n_save == 0) {
        last = k;
        break;
      }
    if (stages) {
      double ts = t;
      for (int k = i; k <= last && !rc; ++k, ts += dt) {
        rc = cupic_charge_deposition(ctx);
        if (!rc) rc = cupic_poisson_solver(ctx, -1.0, 0, 0, 0);
        if (!rc) rc = cupic_field_solver(ctx);
        if (!rc) rc = cupic_particle_mover(ctx);
        if (!rc) rc = cupic_cc(ctx, ts);
      }
    } else {
      rc = cupic_step(ctx, last - i + 1);
      if (!rc) rc = cupic_sync(ctx);
    }
    if (rc) return fail("step", rc);
    for (; i <= last; ++i, t += dt) {
      if (i >= n_prev && i % n_save == 0) {
        rc = snapshot(ctx, out, i);
        if (rc) return fail("snapshot", rc);
      }
      printf("t = %g\n", t);
    }
  }

  rc = cupic_rewrite_input_data(input.c_str(), n_fin);  // main.cu:98-113
  if (rc) return fail("input_data rewrite", rc);
  cupic_destroy(ctx);
  printf("Simulation finished!\n");
  return 0;
}
