// Runs the reference's own particle-file reader and snapshot writers
// (src/init.cu:348-420, src/diagnostic.cu:48-215) on host memory and leaves
// their files in <dir>/output.  TEST INFRASTRUCTURE ONLY.
// Usage: files_main <dir>, where <dir>/input holds input_data,
// particles_in.dat, particles_noheader.dat and mesh.bin (nnx*nny doubles).
#include <cstdio>
#include <string>
#include <vector>
#include <unistd.h>
struct particle {  // stdh.h:30-36
  double x, y, vx, vy;
};
void particles_snapshot(particle *d_p, int *d_bm, std::string filename, double t);
void mesh_snapshot(double *d_m, std::string filename);
void save_bm(int *d_bm, std::string filename);
void save_bins(int *d_bm, particle *d_p, std::string filename);
void read_particle_file(std::string filename, particle **d_p, int **d_bm);
int init_nnx(void);
int init_nny(void);
int main(int argc, char **argv) {
  if (argc < 2) return 2;
  std::string run = std::string(argv[1]) + "/run";
  if (chdir(run.c_str()) != 0) return 3;  // the getters read ../input/input_data
  particle *p = nullptr;
  int *bm = nullptr;
  read_particle_file("../input/particles_in.dat", &p, &bm);
  particles_snapshot(p, bm, "../output/particles_snap", 0.0);
  save_bm(bm, "bm");      // ../output/bm.dat
  save_bins(bm, p, "bins");  // ../output/bins.dat
  read_particle_file("../input/particles_noheader.dat", &p, &bm);
  particles_snapshot(p, bm, "../output/noheader_snap", 0.0);
  const int nn = init_nnx() * init_nny();
  std::vector<double> m(nn);
  FILE *f = std::fopen("../input/mesh.bin", "rb");
  if (!f || std::fread(m.data(), sizeof(double), nn, f) != (size_t)nn) return 4;
  std::fclose(f);
  mesh_snapshot(m.data(), "../output/mesh");
  return 0;
}
