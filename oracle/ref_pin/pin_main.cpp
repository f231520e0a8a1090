// Runs the reference's own input_data getters (src/init.cu:424-789) and
// prints every derived parameter as exact hex doubles.  TEST INFRASTRUCTURE
// ONLY.  Usage: pin_main <dir containing input/input_data>
#include <cstdio>
#include <unistd.h>
#include <string>
double init_qi(void); double init_qe(void); double init_mi(void); double init_me(void);
double init_kti(void); double init_kte(void); double init_phi_p(void); double init_n(void);
double init_Lx(void); double init_Ly(void); double init_ds(void); double init_dt(void);
double init_dtin_i(void); double init_dtin_e(void); double init_epsilon0(void);
int init_ncx(void); int init_ncy(void); int init_nnx(void); int init_nny(void); double init_Dl(void);
int init_n_ini(void); int init_n_prev(void); int init_n_save(void); int init_n_fin(void);
int main(int argc, char **argv) {
  if (argc < 2) return 2;
  std::string run = std::string(argv[1]) + "/run";
  if (chdir(run.c_str()) != 0) return 3;  // the getters read ../input/input_data
  const double n = init_n(), Lx = init_Lx(), ds = init_ds();
  const int ncy = init_ncy();
  const int N = int(n * Lx * ds * ds) * ncy;  // init.cu:136
  std::printf("{\"n\": \"%a\", \"eps0\": \"%a\", \"phi_p\": \"%a\", \"Dl\": \"%a\", \"mi\": \"%a\", "
              "\"kti\": \"%a\", \"me\": \"%a\", \"kte\": \"%a\", \"qe\": \"%a\", \"qi\": \"%a\", "
              "\"ds\": \"%a\", \"dt\": \"%a\", \"Lx\": \"%a\", \"Ly\": \"%a\", \"dtin_e\": \"%a\", "
              "\"dtin_i\": \"%a\", \"ncx\": %d, \"ncy\": %d, \"nnx\": %d, \"nny\": %d, \"n_ini\": %d, "
              "\"n_prev\": %d, \"n_save\": %d, \"n_fin\": %d, \"N\": %d}\n",
              n, init_epsilon0(), init_phi_p(), init_Dl(), init_mi(), init_kti(), init_me(),
              init_kte(), init_qe(), init_qi(), ds, init_dt(), Lx, init_Ly(), init_dtin_e(),
              init_dtin_i(), init_ncx(), ncy, init_nnx(), init_nny(), init_n_ini(), init_n_prev(),
              init_n_save(), init_n_fin(), N);
  return 0;
}
