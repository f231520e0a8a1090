// files.cpp -- the reference's text files: particle and mesh snapshots,
// bookmark and bin dumps, the restart reader and the input_data rewrite
// (src/diagnostic.cu:48-215, src/init.cu:327-420, src/main.cu:98-113).
// The output formats are kept character for character so the reference's
// post-processing reads them unchanged.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "cupic_gpu.h"

namespace {

int close_status(FILE *f) { return fclose(f) == 0 ? CUPIC_OK : CUPIC_ERR_IO; }

// one species in row order, as 4 doubles per particle
int fetch_species(cupic_ctx *ctx, int species, std::vector<double> *buf, int64_t *n) {
  int64_t ne = 0, ni = 0;
  int rc = cupic_get_counts(ctx, &ne, &ni);
  if (rc) return rc;
  const int64_t want = species == 0 ? ne : ni;
  buf->assign((size_t)(4 * (want > 0 ? want : 1)), 0.0);
  return cupic_store_particles(ctx, species, buf->data(), want, n);
}

}  // namespace

extern "C" {

int cupic_write_particles_file(const char *path, const double *xyvv, int64_t n,
                               const char *header) {
  if (!path || n < 0 || (n > 0 && !xyvv)) return CUPIC_ERR_ARG;
  FILE *f = fopen(path, "w");
  if (!f) return CUPIC_ERR_IO;
  if (header) fprintf(f, "# %s\n", header);
  for (int64_t k = 0; k < n; ++k)  // diagnostic.cu:76-79
    fprintf(f, " %.17e %.17e %.17e %.17e \n", xyvv[4 * k], xyvv[4 * k + 1], xyvv[4 * k + 2],
            xyvv[4 * k + 3]);
  return close_status(f);
}

int cupic_read_particles_file(const char *path, double *xyvv, int64_t capacity, int64_t *n_out) {
  if (!path || !n_out || capacity < 0) return CUPIC_ERR_ARG;
  FILE *f = fopen(path, "r");
  if (!f) return CUPIC_ERR_IO;
  std::string line;
  int64_t n = 0;
  int rc = CUPIC_OK;
  char buf[256];
  while (fgets(buf, sizeof buf, f)) {
    line += buf;
    if (line.back() != '\n' && !feof(f)) continue;  // a line longer than buf
    double v[4];
    const int got = sscanf(line.c_str(), " %lf %lf %lf %lf", &v[0], &v[1], &v[2], &v[3]);
    line.clear();
    if (got != 4) continue;
    if (xyvv) {
      if (n >= capacity) {
        rc = CUPIC_ERR_CAPACITY;
        break;
      }
      memcpy(xyvv + 4 * n, v, sizeof v);
    }
    ++n;
  }
  fclose(f);
  *n_out = n;
  return rc;
}

int cupic_write_mesh_file(const char *path, const double *m, int32_t nnx, int32_t nny) {
  if (!path || !m || nnx < 1 || nny < 1) return CUPIC_ERR_ARG;
  FILE *f = fopen(path, "w");
  if (!f) return CUPIC_ERR_IO;
  for (int i = 0; i < nnx; ++i) {  // diagnostic.cu:118-125
    for (int j = 0; j < nny; ++j) fprintf(f, " %d %d %.17e \n", i, j, m[i + (size_t)j * nnx]);
    fprintf(f, "\n");
  }
  return close_status(f);
}

int cupic_write_bookmarks_file(const char *path, const int32_t *bm, int32_t ncy) {
  if (!path || !bm || ncy < 1) return CUPIC_ERR_ARG;
  FILE *f = fopen(path, "w");
  if (!f) return CUPIC_ERR_IO;
  for (int i = 0; i < 2 * ncy; i += 2)  // diagnostic.cu:161-164
    fprintf(f, " %d %d %d \n", i, bm[i], bm[i + 1]);
  return close_status(f);
}

int cupic_write_bins_file(const char *path, const double *xyvv, int64_t n, double ds) {
  if (!path || n < 0 || (n > 0 && !xyvv) || !(ds > 0)) return CUPIC_ERR_ARG;
  FILE *f = fopen(path, "w");
  if (!f) return CUPIC_ERR_IO;
  for (int64_t k = 0; k < n; ++k)  // diagnostic.cu:204-207
    fprintf(f, " %d %d \n", (int)k, (int)(xyvv[4 * k + 1] / ds));
  return close_status(f);
}

int cupic_rewrite_input_data(const char *path, int32_t n_ini) {
  if (!path) return CUPIC_ERR_ARG;
  FILE *f = fopen(path, "r");
  if (!f) return CUPIC_ERR_IO;
  std::vector<std::string> lines(1);
  int ch;
  while ((ch = fgetc(f)) != EOF) {
    lines.back() += (char)ch;
    if (ch == '\n') lines.emplace_back();
  }
  fclose(f);
  if (lines.back().empty()) lines.pop_back();
  if (lines.size() < 2) return CUPIC_ERR_IO;
  lines[1] = "n_ini = " + std::to_string(n_ini) + ";\n";  // main.cu:104
  if (lines.back().back() != '\n') lines.back() += '\n';
  const std::string tmp = std::string(path) + "_new";  // main.cu:99,113
  FILE *o = fopen(tmp.c_str(), "w");
  if (!o) return CUPIC_ERR_IO;
  for (const std::string &l : lines) fputs(l.c_str(), o);
  if (close_status(o)) return CUPIC_ERR_IO;
  return rename(tmp.c_str(), path) == 0 ? CUPIC_OK : CUPIC_ERR_IO;
}

int cupic_particles_snapshot(cupic_ctx *ctx, int species, const char *path) {
  if (!ctx || !path || species < 0 || species > 1) return CUPIC_ERR_ARG;
  std::vector<double> buf;
  int64_t n = 0;
  int rc = fetch_species(ctx, species, &buf, &n);
  if (rc) return rc;
  return cupic_write_particles_file(path, buf.data(), n, nullptr);
}

int cupic_mesh_snapshot(cupic_ctx *ctx, int what, const char *path) {
  if (!ctx || !path || what < 0 || what > 4) return CUPIC_ERR_ARG;
  cupic_params p;
  int rc = cupic_get_params(ctx, &p);
  if (rc) return rc;
  const int nnx = p.ncx + 1, nny = p.ncy + 1;
  std::vector<double> m((size_t)nnx * nny), other((size_t)nnx * nny);
  if (what <= 1)
    rc = cupic_get_rho(ctx, what, m.data());
  else if (what == 2)
    rc = cupic_get_phi(ctx, m.data());
  else if (what == 3)
    rc = cupic_get_field(ctx, m.data(), other.data());
  else
    rc = cupic_get_field(ctx, other.data(), m.data());
  if (rc) return rc;
  return cupic_write_mesh_file(path, m.data(), nnx, nny);
}

int cupic_save_bm(cupic_ctx *ctx, int species, const char *path) {
  if (!ctx || !path || species < 0 || species > 1) return CUPIC_ERR_ARG;
  cupic_params p;
  int rc = cupic_get_params(ctx, &p);
  if (rc) return rc;
  std::vector<int32_t> bm((size_t)2 * p.ncy);
  rc = cupic_get_bookmarks(ctx, species, bm.data());
  if (rc) return rc;
  return cupic_write_bookmarks_file(path, bm.data(), p.ncy);
}

int cupic_save_bins(cupic_ctx *ctx, int species, const char *path) {
  if (!ctx || !path || species < 0 || species > 1) return CUPIC_ERR_ARG;
  cupic_params p;
  int rc = cupic_get_params(ctx, &p);
  if (rc) return rc;
  std::vector<double> buf;
  int64_t n = 0;
  rc = fetch_species(ctx, species, &buf, &n);
  if (rc) return rc;
  return cupic_write_bins_file(path, buf.data(), n, p.ds);
}

int cupic_load_particles_file(cupic_ctx *ctx, int species, const char *path) {
  if (!ctx || !path || species < 0 || species > 1) return CUPIC_ERR_ARG;
  int64_t n = 0;
  int rc = cupic_read_particles_file(path, nullptr, 0, &n);
  if (rc) return rc;
  std::vector<double> buf((size_t)(4 * (n > 0 ? n : 1)));
  int64_t got = 0;
  rc = cupic_read_particles_file(path, buf.data(), n, &got);
  if (rc) return rc;
  return cupic_load_particles(ctx, species, buf.data(), got);
}

}  // extern "C"
