// capi.cu -- the extern "C" entry points of libcupic_gpu.so.
//
// A cupic_ctx owns the device state of one plasma slab.  The stage entry
// points mirror the reference's host functions (include/cupic_gpu.h lists
// each with its file:line); cupic_step runs whole cycles from a captured
// CUDA graph.  Errors are returned as CUPIC_* codes, never by exit().
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <new>
#include <tuple>
#include <vector>

#include "ctx.h"
#include "kernels.h"

using namespace cupic;

cudaError_t cupic::raise_dyn_smem(const void *kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, size_t> cur;
  if (bytes <= 48 * 1024) return cudaSuccess;  // below the default limit
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  size_t &have = cur[std::make_pair(kernel, dev)];
  if (bytes <= have) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) have = bytes;
  return e;
}

namespace {

#define CU(call)                                 \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

// waits for the context's work, completing a run that ran out of room
#define SETTLE(c)              \
  do {                         \
    const int rc_ = settle(c); \
    if (rc_) return rc_;       \
  } while (0)

int cuda_status(cudaError_t e) {
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    return CUPIC_ERR_NOMEM;
  }
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return CUPIC_ERR_NODEVICE;
  return CUPIC_ERR_CUDA;
}

// A context's device memory comes from the device's stream-ordered pool,
// allocated and freed in the order of the context's stream: creating or
// destroying a context never waits for the device (other contexts may be
// stepping), and a server reuses the memory of finished requests.
template <class T>
cudaError_t dalloc(cupic_ctx *c, T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  return cudaMallocAsync((void **)p, n * sizeof(T), c->stream);
}

void dfree(cupic_ctx *c, void *p) {
  if (p) cudaFreeAsync(p, c->stream);
}

// the default pool keeps freed memory for the next allocation instead of
// returning it to the system at every synchronisation
cudaError_t keep_pool(int device) {
  cudaMemPool_t pool;
  cudaError_t e = cudaDeviceGetDefaultMemPool(&pool, device);
  if (e != cudaSuccess) return e;
  uint64_t keep = UINT64_MAX;
  return cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
}

// The device address of a host buffer that kernels can read in place
// (page-locked and mapped: cudaHostAlloc, cudaHostRegister, a pinned
// framework tensor), or null for pageable memory, which is staged instead.
void *mapped_host(const void *p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// `bytes` of the context's transfer scratch (grown, never shrunk: repeated
// uploads and downloads allocate nothing)
cudaError_t io_scratch(cupic_ctx *c, size_t bytes, void **out) {
  if (bytes > c->io_cap) {
    dfree(c, c->io_buf);
    c->io_buf = nullptr;
    c->io_cap = 0;
    cudaError_t e = dalloc(c, reinterpret_cast<unsigned char **>(&c->io_buf), bytes);
    if (e != cudaSuccess) return e;
    c->io_cap = bytes;
  }
  *out = c->io_buf;
  return cudaSuccess;
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

// The streams and events of destroyed contexts, kept per device for the
// next contexts: creating a stream can stall for tens of milliseconds while
// the device is busy, which a server admitting requests cannot afford.
struct StreamSet {
  cudaStream_t stream, side;
  cudaEvent_t fork, join;
};
std::mutex g_streams_mu;
std::vector<std::vector<StreamSet>> g_streams;

cudaError_t new_stream_set(StreamSet *s) {
  *s = {};
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming);
  return e;
}

void keep_stream_set(int device, const StreamSet &s) {
  std::lock_guard<std::mutex> lk(g_streams_mu);
  if ((int)g_streams.size() <= device) g_streams.resize(device + 1);
  g_streams[device].push_back(s);
}

cudaError_t take_stream_set(int device, StreamSet *s) {
  {
    std::lock_guard<std::mutex> lk(g_streams_mu);
    if ((int)g_streams.size() > device && !g_streams[device].empty()) {
      *s = g_streams[device].back();
      g_streams[device].pop_back();
      return cudaSuccess;
    }
  }
  return new_stream_set(s);
}

int32_t round8(double v) { return (int32_t)((((int64_t)ceil(v)) + 7) / 8 * 8); }

void free_species(cupic_ctx *c, SpeciesDev &S) {
  dfree(c, S.parts);
  dfree(c, S.seg);
  dfree(c, S.cap);
  dfree(c, S.cnt);
  dfree(c, S.nstay);
  dfree(c, S.nup);
  dfree(c, S.ndown);
  dfree(c, S.stage_up);
  dfree(c, S.stage_down);
  dfree(c, S.inj_tin);
  dfree(c, S.inj_p);
  dfree(c, S.inj_d);
  memset(&S, 0, sizeof(S));
}

void destroy_graph(cupic_ctx *c) {
  if (c->graph) cudaGraphExecDestroy(c->graph);
  c->graph = nullptr;
  c->graph_ok = false;
}

// (Re)allocates one species with row capacities cap[j]; live counts are 0.
int layout_species(cupic_ctx *c, int sp, const std::vector<int32_t> &capv) {
  SpeciesDev &S = c->a.sp[sp];
  const int ncy = c->p.ncy;
  const int inj_cap = S.inj_cap;
  free_species(c, S);
  S.inj_cap = inj_cap;
  c->cap[sp] = capv;
  c->seg[sp].assign(ncy, 0);
  int64_t tot = 0;
  int32_t cmax = 0;
  for (int j = 0; j < ncy; ++j) {
    c->seg[sp][j] = tot;
    tot += capv[j];
    cmax = std::max(cmax, capv[j]);
  }
  c->total_cap[sp] = tot;
  S.stage_cap = round8(cmax * c->p.stage_frac) + 64;
  CU(dalloc(c, &S.parts, (size_t)tot));
  CU(dalloc(c, &S.seg, ncy));
  CU(dalloc(c, &S.cap, ncy));
  CU(dalloc(c, &S.cnt, ncy));
  CU(dalloc(c, &S.nstay, ncy));
  CU(dalloc(c, &S.nup, ncy));
  CU(dalloc(c, &S.ndown, ncy));
  CU(dalloc(c, &S.stage_up, (size_t)ncy * S.stage_cap));
  CU(dalloc(c, &S.stage_down, (size_t)ncy * S.stage_cap));
  CU(dalloc(c, &S.inj_tin, (size_t)S.inj_cap));
  CU(dalloc(c, &S.inj_p, (size_t)S.inj_cap));
  CU(dalloc(c, &S.inj_d, (size_t)S.inj_cap));
  const bool uniform = std::all_of(capv.begin(), capv.end(), [&](int32_t v) { return v == capv[0]; });
  if (uniform) {
    // filled on the context's stream: no host wait
    CU(launch_uniform_layout(S, ncy, capv.empty() ? 0 : capv[0], c->stream));
  } else {
    CU(cudaStreamSynchronize(c->stream));
    CU(cudaMemcpy(S.seg, c->seg[sp].data(), ncy * sizeof(int64_t), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(S.cap, capv.data(), ncy * sizeof(int32_t), cudaMemcpyHostToDevice));
    CU(cudaMemset(S.cnt, 0, ncy * sizeof(int32_t)));
    CU(cudaMemset(S.nstay, 0, ncy * sizeof(int32_t)));
    CU(cudaMemset(S.nup, 0, ncy * sizeof(int32_t)));
    CU(cudaMemset(S.ndown, 0, ncy * sizeof(int32_t)));
    CU(cudaDeviceSynchronize());
  }
  destroy_graph(c);
  ++c->layout_epoch;  // a batch holding this context's SimArgs rebuilds
  return CUPIC_OK;
}

int validate(const cupic_params *p) {
  if (!p) return CUPIC_ERR_ARG;
  if (p->ncx < 2 || p->ncy < 2 || p->ncx > 4096 || p->ncy > (1 << 20)) return CUPIC_ERR_ARG;
  if (!(p->ds > 0) || !(p->dt > 0) || !(p->n > 0) || !(p->eps0 > 0)) return CUPIC_ERR_ARG;
  if (!(p->me > 0) || !(p->mi > 0) || !(p->kte > 0) || !(p->kti > 0)) return CUPIC_ERR_ARG;
  if (p->ppr < 0 || p->max_sweeps < 0 || p->init_max_sweeps < 0) return CUPIC_ERR_ARG;
  if (!(p->row_slack >= 0) || !(p->stage_frac > 0)) return CUPIC_ERR_ARG;
  return CUPIC_OK;
}

void fill_constants(cupic_ctx *c) {
  const cupic_params &p = c->p;
  SimArgs &a = c->a;
  a.ncx = p.ncx;
  a.ncy = p.ncy;
  a.nnx = p.ncx + 1;
  a.nny = p.ncy + 1;
  const double Lxd = p.ds * p.ncx, Lyd = p.ds * p.ncy;
  a.ds = (float)p.ds;
  a.inv_ds = (float)(1.0 / p.ds);
  a.Lx = (float)Lxd;
  a.Ly = (float)Lyd;
  a.two_ds = (float)(2.0 * p.ds);
  a.dt = (float)p.dt;
  const double q[2] = {p.qe, p.qi}, m[2] = {p.me, p.mi}, kt[2] = {p.kte, p.kti};
  for (int s = 0; s < 2; ++s) {
    a.dtqm[s] = (float)(p.dt * q[s] / m[s]);
    a.mhdtqm[s] = (float)(-0.5 * p.dt * q[s] / m[s]);
    a.qm[s] = q[s] / m[s];
    a.sig[s] = sqrt(kt[s] / m[s]);
    /* init.cu:686-714 */
    a.dtin[s] = sqrt(2.0 * 3.1415926535897932 * m[s] / kt[s]) / (p.n * Lxd * p.ds);
  }
  a.ds_d = p.ds;
  a.inv_ds_d = 1.0 / p.ds;
  a.Lx_d = Lxd;
  a.Ly_d = Lyd;
  a.dt_d = p.dt;
  a.cb = ldexp(1.0, -32) / (p.ds * p.eps0);
  a.ppr = p.ppr;
  a.k0 = (uint32_t)p.seed;
  a.k1 = (uint32_t)(p.seed >> 32);
}

JacobiArgs jargs(const cupic_ctx *c, double tol, int mn, int mx, int chk, int field);

// ---- Jacobi layout -------------------------------------------------------
// G CTAs of 512 threads, each holding its B mesh rows plus K halo rows on
// each side in shared memory; neighbours trade K rows every K sweeps.  The
// layout changes only the speed: every plan computes the same bits.

// Padded row pitch (16-byte rows) and the rows one CTA's shared memory holds.
void jacobi_geometry(const cupic_ctx *c, int dev_max, int *P, long long *rows_fit) {
  *P = (c->a.nnx + 3) / 4 * 4;
  const size_t avail = (size_t)dev_max - 1024;  // static shared memory of the kernel
  *rows_fit = (long long)(avail / (3 * sizeof(float) * (size_t)*P));
}

// Rows per CTA for G CTAs at depth K, or 0 if the layout does not fit.
int jacobi_rows(const cupic_ctx *c, int G, int K, int P, long long rows_fit) {
  const int M = c->a.nny - 2;
  if (G < 1 || G > M || K < 1) return 0;
  const int B = (M + G - 1) / G;
  if (G > 1 && K > M / G) return 0;  // a CTA sends K of its own rows (it owns >= M/G)
  if (B + 2 * (G > 1 ? K : 1) > rows_fit) return 0;
  int per_sm = 0;
  if (jacobi_set_smem(jacobi_smem_bytes(B, G > 1 ? K : 1, P)) != cudaSuccess ||
      jacobi_max_ctas(jacobi_smem_bytes(B, G > 1 ? K : 1, P), &per_sm) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (per_sm < 1 || G > per_sm * c->num_sms) return 0;
  return B;
}

int alloc_jacobi_scratch(cupic_ctx *c, int G, long long GK, int P) {
  dfree(c, c->jflags);
  dfree(c, c->jres);
  dfree(c, c->jhalo);
  c->jflags = nullptr;
  c->jres = nullptr;
  c->jhalo = nullptr;
  CU(dalloc(c, &c->jflags, (size_t)G + 1));
  CU(dalloc(c, &c->jres, (size_t)2 * G));
  CU(dalloc(c, &c->jhalo, (size_t)4 * GK * P));
  c->jhalo_words = (size_t)4 * GK * P;
  // epoch 0 is never valid; the solves on the context's stream follow the clearing
  CU(cudaMemsetAsync(c->jhalo, 0, sizeof(unsigned long long) * c->jhalo_words, c->stream));
  c->epoch_solves = 0;
  return CUPIC_OK;
}

// A halo word carries the epoch (solve count << 16) + exchange index in 32
// bits, so the solve count wraps every 65,536 solves.  A slot that the
// solves since stopped rewriting (tolerance-stopped solves end after
// different numbers of exchanges) could then hold a word whose epoch matches
// again.  Before `solves` more solves are enqueued, the halo words are
// zeroed (epoch 0 never matches) whenever the count since the last clearing
// would reach kEpochGuard, ordered on the context's stream before them.
constexpr int64_t kEpochGuard = 65000;
int epoch_guard(cupic_ctx *c, int64_t solves) {
  if (c->jhalo && c->epoch_solves + solves > kEpochGuard) {
    CU(cudaMemsetAsync(c->jhalo, 0, sizeof(unsigned long long) * c->jhalo_words, c->stream));
    c->epoch_solves = 0;
  }
  c->epoch_solves += solves;
  return CUPIC_OK;
}

// solves (Jacobi launches) one solve of at most mx sweeps enqueues
int64_t solves_of(const cupic_ctx *c, int mx) {
  const int m = c->p.refine_every;
  return m > 0 ? 1 + (std::max(mx, 0) + m - 1) / m : 1;
}

int set_jacobi_plan(cupic_ctx *c, int G, int B, int K, int P) {
  c->jG = G;
  c->jB = B;
  c->jK = G > 1 ? K : 1;
  c->jP = P;
  CU(jacobi_set_smem(jacobi_smem_bytes(B, c->jK, P)));
  return alloc_jacobi_scratch(c, G, (long long)G * c->jK, P);
}

// The fixed rule, used when tuning is off or a layout is forced with
// CUPIC_JACOBI_CTAS / CUPIC_JACOBI_DEPTH: one CTA for small meshes or
// frequent convergence checks (each check of a multi-CTA solve is a grid
// barrier), else one CTA per SM with the deepest halo that fits.
int plan_jacobi_rule(cupic_ctx *c, int P, long long rows_fit) {
  const int M = c->a.nny - 2, nnx = c->a.nnx;
  const char *env = getenv("CUPIC_JACOBI_CTAS");
  const char *envk = getenv("CUPIC_JACOBI_DEPTH");
  int G = env ? atoi(env) : 0;
  int K = envk ? atoi(envk) : 0;
  if (G <= 0) {
    const bool fits = M + 2 <= rows_fit;
    const bool frequent_checks = c->p.check_every < 16 && c->p.max_sweeps > c->p.min_sweeps;
    if (fits && ((long long)M * nnx <= 65536 || frequent_checks))
      G = 1;
    else
      G = std::min(c->num_sms, M);
  }
  G = std::max(1, std::min(G, M));
  int B = (M + G - 1) / G;
  if (K <= 0) K = 16;
  K = std::max(1, std::min(K, std::min(M / G, 16)));
  if (G == 1) K = 1;
  while (G > 1 && B + 2 * K > rows_fit) {  // shrink the depth, then add CTAs
    if (K > 1) {
      --K;
    } else {
      ++G;
      B = (M + G - 1) / G;
    }
  }
  if (B + 2 * K > rows_fit) return CUPIC_ERR_ARG;
  if (!jacobi_rows(c, G, K, P, rows_fit)) return CUPIC_ERR_ARG;
  return set_jacobi_plan(c, G, B, K, P);
}

// Autotuner: times every feasible (CTAs, depth) layout on this context's own
// buffers for the solve it will run (its check interval, up to 256 sweeps,
// with the field) and keeps the fastest.  Results are cached per device and
// mesh shape, so contexts of one shape tune once per process.
struct TuneKey {
  int device, nnx, nny, chk, sweeps;
  bool operator<(const TuneKey &o) const {
    return std::tie(device, nnx, nny, chk, sweeps) < std::tie(o.device, o.nnx, o.nny, o.chk, o.sweeps);
  }
};
std::mutex g_tune_mu;
struct TunePick {
  int G, K;
  bool nostrip;
};
std::map<TuneKey, TunePick> g_tuned;

int tune_jacobi(cupic_ctx *c, int P, long long rows_fit) {
  const int M = c->a.nny - 2;
  const int chk = std::max(1, c->p.check_every);
  const int S = std::max(1, std::min(std::max(c->p.max_sweeps, c->p.init_max_sweeps), 256));
  const TuneKey key{c->device, c->a.nnx, c->a.nny, chk, S};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      const int G = it->second.G, K = it->second.K;
      const int B = jacobi_rows(c, G, K, P, rows_fit);
      c->jNoStrip = it->second.nostrip;
      if (B) return set_jacobi_plan(c, G, B, K, P);
    }
  }
  // every layout is timed with the sweep form it would get, and again with
  // the shared-memory sweep where that form is register strips
  struct Cand { int G, B, K; bool nostrip; };
  std::vector<Cand> cands;
  const int ns = c->num_sms;
  const int gs[] = {1, 2, 4, 8, 16, 24, ns / 4, ns / 2, ns};
  int maxG = 1;
  long long maxGK = 1;
  for (int G : gs) {
    if (G < 1 || G > M) continue;
    if (!cands.empty() && cands.back().G == G) continue;
    // powers of two and the deepest halo that fits
    int kmax = G == 1 ? 1 : std::min(16, M / G);
    while (kmax > 1 && !jacobi_rows(c, G, kmax, P, rows_fit)) --kmax;
    for (int K : {1, 2, 4, 8, 16, kmax}) {
      if (K > kmax) continue;
      if (!cands.empty() && cands.back().G == G && cands.back().K >= K) continue;  // no repeats
      const int B = jacobi_rows(c, G, K, P, rows_fit);
      if (!B) continue;
      cands.push_back({G, B, K, false});
      if (jacobi_strip_rows(c->a.nnx, B + 2 * (G > 1 ? K : 1) - 2) > 0) cands.push_back({G, B, K, true});
      maxG = std::max(maxG, G);
      maxGK = std::max(maxGK, (long long)G * K);
    }
  }
  if (cands.empty()) return plan_jacobi_rule(c, P, rows_fit);
  int rc = alloc_jacobi_scratch(c, maxG, maxGK, P);
  if (rc) return rc;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  float best = 1e30f;
  Cand pick = cands.front();
  for (const Cand &cd : cands) {
    c->jG = cd.G;
    c->jB = cd.B;
    c->jK = cd.G > 1 ? cd.K : 1;
    c->jP = P;
    c->jNoStrip = cd.nostrip;
    // write_stats keeps the residual checks of the real solve (a solve with
    // no tolerance that reports nothing skips them); the stats it writes
    // are overwritten by the first real solve
    JacobiArgs J = jargs(c, 0.0, S, S, chk, 1);
    J.write_stats = 1;
    float t = 1e30f;
    bool ok = true;
    for (int rep = 0; rep < 3 && ok; ++rep) {
      ok = cudaEventRecord(e0, c->stream) == cudaSuccess &&
           launch_jacobi(c->a, J, c->stream) == cudaSuccess &&
           cudaEventRecord(e1, c->stream) == cudaSuccess &&
           cudaEventSynchronize(e1) == cudaSuccess;
      float ms = 0.0f;
      if (ok && rep > 0 && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) t = std::min(t, ms);
    }
    if (!ok) {
      cudaGetLastError();
      continue;
    }
    if (t < best) {
      best = t;
      pick = cd;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // a solve that gave up waiting leaves a flag: clear what the trials raised
  CU(cudaMemsetAsync(&c->ctl->step_flags, 0, sizeof(uint32_t), c->stream));
  CU(cudaStreamSynchronize(c->stream));
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[key] = {pick.G, pick.K, pick.nostrip};
  }
  c->jNoStrip = pick.nostrip;
  return set_jacobi_plan(c, pick.G, pick.B, pick.K, P);
}

int plan_jacobi(cupic_ctx *c) {
  int dev_max = 0;
  CU(cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
  int P = 0;
  long long rows_fit = 0;
  jacobi_geometry(c, dev_max, &P, &rows_fit);
  const char *tune = getenv("CUPIC_JACOBI_TUNE");
  if (getenv("CUPIC_JACOBI_CTAS") || getenv("CUPIC_JACOBI_DEPTH") || (tune && atoi(tune) == 0))
    return plan_jacobi_rule(c, P, rows_fit);
  return tune_jacobi(c, P, rows_fit);
}

JacobiArgs jargs(const cupic_ctx *c, double tol, int mn, int mx, int chk, int field) {
  JacobiArgs J{};
  J.tol = tol;
  J.min_sweeps = mn;
  J.max_sweeps = mx;
  J.check_every = chk < 1 ? 1 : chk;
  J.G = c->jG;
  J.rows_per_cta = c->jB;
  J.depth = c->jK;
  J.pitch = c->jP;
  J.vec = ((c->a.nnx - 1) % 4 == 0) ? 1 : 0;
  J.strip = jacobi_strip_rows(c->a.nnx, c->jB + 2 * (c->jG > 1 ? c->jK : 1) - 2);
  if (getenv("CUPIC_JACOBI_SCALAR")) J.vec = 0;
  if (c->jNoStrip || getenv("CUPIC_JACOBI_SCALAR") || getenv("CUPIC_JACOBI_NOSTRIP")) J.strip = 0;
  J.do_field = field;
  J.write_stats = 1;
  J.flags = c->jflags;
  J.bar = c->jflags + c->jG;
  J.res_cta = c->jres;
  J.halo = c->jhalo;
  return J;
}

int set_phi_both(cupic_ctx *c, const double *phi) {
  const size_t n = (size_t)c->a.nnx * c->a.nny;
  CU(cudaStreamSynchronize(c->stream));  // no kernel of the context still uses phi
  std::vector<float> h(n);
  for (size_t k = 0; k < n; ++k) h[k] = (float)phi[k];
  CU(cudaMemcpy(c->a.phi, h.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  if (c->phi64) CU(cudaMemcpy(c->phi64, phi, n * sizeof(double), cudaMemcpyHostToDevice));
  return CUPIC_OK;
}

int set_linear_phi(cupic_ctx *c) {  // init.cu:235-241, on the device
  CU(launch_linear_phi(c->a, c->p.phi_p, c->phi64, c->stream));
  return CUPIC_OK;
}

// Precision form (refine_every = m > 0): every m FP32 Jacobi sweeps on the
// correction, an FP64 residual and update; stops when the residual's max
// norm is below tol after at least mn sweeps, or at mx sweeps.  The host
// reads the norm once per m sweeps.
int refine_solve(cupic_ctx *c, double tol, int mn, int mx, int field, int write_stats) {
  const int m = c->p.refine_every;
  unsigned long long *hbits = static_cast<unsigned long long *>(c->h_pin);
  int sweeps = 0;
  double res = 0.0;
  CU(launch_r64_source(c->a, c->b64, c->stream));
  for (;;) {
    CU(launch_r64_residual(c->a, c->phi64, c->b64, c->rr, c->maxr, c->stream));
    CU(cudaMemcpyAsync(hbits, c->maxr, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                       c->stream));
    CU(cudaStreamSynchronize(c->stream));
    memcpy(&res, hbits, sizeof(double));
    if ((sweeps >= mn && res < tol) || sweeps >= mx) break;
    const int k = std::min(m, mx - sweeps);
    JacobiArgs J = jargs(c, 0.0, k, k, k, 0);
    J.write_stats = 0;
    J.phi = c->dl;  // the correction starts from zero
    J.phi_zero = 1;
    J.src = c->rr;
    CU(launch_jacobi(c->a, J, c->stream));
    CU(launch_r64_update(c->a, c->phi64, c->dl, c->stream));
    sweeps += k;
  }
  // the FP32 potential (and the field) from phi64
  if (field) CU(launch_r64_field(c->a, c->phi64, c->stream));
  else CU(launch_r64_phi32(c->a, c->phi64, c->stream));
  if (write_stats) {
    struct {
      int32_t sweeps;
      float residual;
    } st = {sweeps, (float)res};
    static_assert(offsetof(Ctl, residual) == offsetof(Ctl, sweeps) + 4, "Ctl layout");
    memcpy(hbits + 1, &st, sizeof(st));
    CU(cudaMemcpyAsync(&c->ctl->sweeps, hbits + 1, sizeof(st), cudaMemcpyHostToDevice, c->stream));
  }
  return CUPIC_OK;
}

// The same solve with the stop test on the device: every correction of the
// sweep cap is enqueued, and once the test has passed the remaining ones
// return at once.  Nothing waits on the host, so a step in the precision
// form is captured as one graph.  Each correction is one Jacobi launch with
// the residual, the test and the update fused in (JacobiArgs::r64_phi): the
// operations and their order are those of refine_solve's separate kernels,
// so the results are identical, with three launches and two passes over
// the FP64 potential fewer per correction.  A last launch without sweeps
// tests the residual after the final correction.  Caps needing more than
// kDeviceCorrections corrections use refine_solve.
constexpr int kDeviceCorrections = 512;

bool refine_on_device(const cupic_ctx *c, int mx) {
  const int m = c->p.refine_every;
  return (long long)(std::max(mx, 0) + m - 1) / m <= kDeviceCorrections;
}

int refine_solve_device(cupic_ctx *c, double tol, int mn, int mx, int field, int write_stats) {
  const int m = c->p.refine_every;
  CU(cudaMemsetAsync(&c->ctl->refine_done, 0, sizeof(int32_t), c->stream));
  CU(launch_r64_source(c->a, c->b64, c->stream));
  for (int sweeps = 0;;) {
    const int k = sweeps >= mx ? 0 : std::min(m, mx - sweeps);
    JacobiArgs J = jargs(c, 0.0, k, k, std::max(k, 1), 0);
    J.write_stats = 0;
    J.phi = c->dl;  // the correction starts from zero
    J.phi_zero = 1;
    J.gated = 1;
    J.r64_phi = c->phi64;
    J.r64_b = c->b64;
    J.r64_tol = tol;
    J.r64_done = sweeps;
    J.r64_mn = mn;
    J.r64_mx = mx;
    J.r64_stats = write_stats;
    CU(launch_jacobi(c->a, J, c->stream));
    if (sweeps >= mx) break;
    sweeps += k;
  }
  // the FP32 potential (and the field) from phi64
  if (field) CU(launch_r64_field(c->a, c->phi64, c->stream));
  else CU(launch_r64_phi32(c->a, c->phi64, c->stream));
  return CUPIC_OK;
}

// the solve of a step or stage call, FP32 or in the precision form
int run_solve(cupic_ctx *c, double tol, int mn, int mx, int chk, int field, int write_stats = 1) {
  if (c->p.refine_every > 0)
    return refine_on_device(c, mx) ? refine_solve_device(c, tol, mn, mx, field, write_stats)
                                   : refine_solve(c, tol, mn, mx, field, write_stats);
  JacobiArgs J = jargs(c, tol, mn, mx, chk, field);
  J.write_stats = write_stats;
  CU(launch_jacobi(c->a, J, c->stream));
  return CUPIC_OK;
}

// a step's solve, which also clears the next charge accumulator (the
// precision form's solve does not: the step clears it separately)
int run_step_solve(cupic_ctx *c, bool *zeroed) {
  const cupic_params &p = c->p;
  *zeroed = false;
  if (p.refine_every > 0) return run_solve(c, p.tol, p.min_sweeps, p.max_sweeps, p.check_every, 1);
  JacobiArgs J = jargs(c, p.tol, p.min_sweeps, p.max_sweeps, p.check_every, 1);
  J.zero_next = 1;
  CU(launch_jacobi(c->a, J, c->stream));
  *zeroed = true;
  return CUPIC_OK;
}

int deposit_current(cupic_ctx *c) {
  CU(cudaMemsetAsync(c->a.rho[c->host_cur], 0,
                     sizeof(unsigned long long) * (size_t)c->a.nnx * c->a.nny, c->stream));
  CU(launch_deposit(c->a, c->stream));
  c->rho_valid = true;
  return CUPIC_OK;
}

int sync_check(cupic_ctx *c) {
  CU(cudaStreamSynchronize(c->stream));
  CU(cudaGetLastError());
  return CUPIC_OK;
}

int read_ctl_flags(cupic_ctx *c, uint32_t *out) {
  uint32_t f[2];
  CU(cudaMemcpy(f, &c->ctl->flags, sizeof(f), cudaMemcpyDeviceToHost));
  *out = f[0] | f[1] | c->host_flags;
  return CUPIC_OK;
}

// status for flags raised on the device
int flag_status(uint32_t f) {
  if (f & CUPIC_FLAG_TIMEOUT) return CUPIC_ERR_TIMEOUT;
  if (f & (CUPIC_FLAG_CAPACITY | CUPIC_FLAG_STAGE)) return CUPIC_ERR_CAPACITY;
  if (f & CUPIC_FLAG_NONFINITE) return CUPIC_ERR_NONFINITE;
  if (f & (CUPIC_FLAG_CFL | CUPIC_FLAG_XRANGE)) return CUPIC_ERR_CFL;
  return CUPIC_OK;
}

int settle(cupic_ctx *c);

int finish(cupic_ctx *c) {
  int rc = settle(c);
  if (rc) return rc;
  rc = sync_check(c);
  if (rc) return rc;
  uint32_t f = 0;
  rc = read_ctl_flags(c, &f);
  if (rc) return rc;
  return flag_status(f);
}

// One step: solve + field, then the injection draws on the side stream while
// the main stream clears the next charge, pushes and appends the movers;
// the injected particles are appended once both branches are done.
// marks: null, or CUPIC_NPHASE events recorded on the main stream after the
// solve, the clearing, the push, the arrivals (with the wait for the draws
// and the room check), the append and the bookkeeping -- the phases of
// cupic_step_timed.
int enqueue_after_solve(cupic_ctx *c, bool zeroed, const cudaEvent_t *marks = nullptr) {
  auto mark = [&](int k) { return marks ? cudaEventRecord(marks[k], c->stream) : cudaSuccess; };
  CU(mark(0));
  CU(cudaEventRecord(c->ev_fork, c->stream));
  CU(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
  CU(launch_inject_draw(c->a, c->side));
  CU(cudaEventRecord(c->ev_join, c->side));
  if (!zeroed) CU(launch_zero_next_rho(c->a, c->stream));
  CU(mark(1));
  CU(launch_push_deposit(c->a, c->stream));
  CU(mark(2));
  CU(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
  CU(launch_room(c->a, c->stream));
  CU(launch_arrive(c->a, c->stream));
  CU(mark(3));
  CU(launch_inject_append(c->a, c->stream));
  CU(mark(4));
  CU(launch_finalize(c->a, c->stream));
  CU(mark(5));
  return CUPIC_OK;
}

int enqueue_step(cupic_ctx *c, const cudaEvent_t *marks = nullptr) {
  bool zeroed = false;
  int rc = run_step_solve(c, &zeroed);
  if (rc) return rc;
  return enqueue_after_solve(c, zeroed, marks);
}

int capture_step(cupic_ctx *c) {
  destroy_graph(c);
  cudaGraph_t g = nullptr;
  CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  const int rc = enqueue_step(c);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (rc != CUPIC_OK || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    c->graph_ok = false;
    return CUPIC_OK;  // fall back to direct launches
  }
  e = cudaGraphInstantiate(&c->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();
    c->graph = nullptr;
    c->graph_ok = false;
    return CUPIC_OK;
  }
  c->graph_ok = true;
  return CUPIC_OK;
}

// n steps, graph-launched where the step is captured
int launch_steps(cupic_ctx *c, int64_t n) {
  if (n <= 0) return CUPIC_OK;
  if (!c->graph_ok) {
    int rc = capture_step(c);
    if (rc) return rc;
  }
  for (int64_t i = 0; i < n; ++i) {
    int rc = epoch_guard(c, solves_of(c, c->p.max_sweeps));
    if (rc) return rc;
    if (c->graph_ok) {
      CU(cudaGraphLaunch(c->graph, c->stream));
    } else {
      int rc = enqueue_step(c);
      if (rc) return rc;
    }
    c->host_cur ^= 1;
  }
  return CUPIC_OK;
}

// ---------------------------------------------------------------------------
// rows that run out of room (the room check of particles.cu halts the run)
// ---------------------------------------------------------------------------
int read_i32(const int32_t *src, int64_t n, std::vector<int32_t> &out) {
  out.assign((size_t)std::max<int64_t>(n, 0), 0);
  if (n > 0) CU(cudaMemcpy(out.data(), src, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost));
  return CUPIC_OK;
}

// Gives every row j of species sp that cannot hold need[j] particles the
// capacity need[j] * (1 + row_slack) + 64, in a new particle array, and
// moves the first keep[j] particles of every row (keep: a device array)
// there in order.  Other rows keep their capacity.  The stream is idle.
int fit_rows(cupic_ctx *c, int sp, const std::vector<int64_t> &need, const int32_t *keep) {
  SpeciesDev &S = c->a.sp[sp];
  const int ncy = c->p.ncy;
  std::vector<int32_t> capv = c->cap[sp];
  bool grow = false;
  for (int j = 0; j < ncy; ++j)
    if (need[j] > capv[j]) {
      const double want = (double)need[j] * (1.0 + c->p.row_slack) + 64.0;
      if (want > 2.0e9) return CUPIC_ERR_CAPACITY;
      capv[j] = round8(want);
      grow = true;
    }
  if (!grow) return CUPIC_OK;
  std::vector<int64_t> seg(ncy);
  int64_t tot = 0;
  for (int j = 0; j < ncy; ++j) {
    seg[j] = tot;
    tot += capv[j];
  }
  float4 *parts = nullptr;
  int64_t *dseg = nullptr;
  int32_t *dcap = nullptr;
  cudaError_t e = dalloc(c, &parts, (size_t)tot);
  if (e == cudaSuccess) e = dalloc(c, &dseg, (size_t)ncy);
  if (e == cudaSuccess) e = dalloc(c, &dcap, (size_t)ncy);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dseg, seg.data(), ncy * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dcap, capv.data(), ncy * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = launch_move_rows(S.parts, S.seg, parts, dseg, keep, ncy, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {  // the old layout stays
    dfree(c, parts);
    dfree(c, dseg);
    dfree(c, dcap);
    cudaStreamSynchronize(c->stream);
    return cuda_status(e);
  }
  dfree(c, S.parts);
  dfree(c, S.seg);
  dfree(c, S.cap);
  S.parts = parts;
  S.seg = dseg;
  S.cap = dcap;
  c->cap[sp] = capv;
  c->seg[sp] = seg;
  c->total_cap[sp] = tot;
  destroy_graph(c);  // the captured launches hold the old pointers
  ++c->layout_epoch;
  return CUPIC_OK;
}

// staging rows sized for the largest row, once the staged movers of the
// running step have arrived (the frees are ordered after the arrivals)
int fit_staging(cupic_ctx *c, int sp) {
  SpeciesDev &S = c->a.sp[sp];
  const int ncy = c->p.ncy;
  const int32_t cmax = c->cap[sp].empty() ? 0 : *std::max_element(c->cap[sp].begin(), c->cap[sp].end());
  const int32_t want = round8(cmax * c->p.stage_frac) + 64;
  if (want <= S.stage_cap) return CUPIC_OK;
  float4 *up = nullptr, *down = nullptr;
  cudaError_t e = dalloc(c, &up, (size_t)ncy * want);
  if (e == cudaSuccess) e = dalloc(c, &down, (size_t)ncy * want);
  if (e != cudaSuccess) {  // the old staging rows stay
    dfree(c, up);
    return cuda_status(e);
  }
  dfree(c, S.stage_up);
  dfree(c, S.stage_down);
  S.stage_up = up;
  S.stage_down = down;
  S.stage_cap = want;
  destroy_graph(c);
  ++c->layout_epoch;
  return CUPIC_OK;
}

// A run halted by the room check: the halted step has pushed and deposited,
// its movers sit in the staging rows and its injected particles in inj_p.
// Grow the rows that cannot take them, complete the step, then run the
// steps that returned at once (skipped counts the halted step too).
int complete_halted(cupic_ctx *c, int32_t skipped) {
  const int ncy = c->p.ncy;
  int32_t ne[2] = {0, 0};
  CU(cudaMemcpy(ne, c->ctl->inj_gen, sizeof(ne), cudaMemcpyDeviceToHost));
  for (int sp = 0; sp < 2; ++sp) {
    const SpeciesDev &S = c->a.sp[sp];
    std::vector<int32_t> ns, nu, nd, dst;
    int rc = read_i32(S.nstay, ncy, ns);
    if (!rc) rc = read_i32(S.nup, ncy, nu);
    if (!rc) rc = read_i32(S.ndown, ncy, nd);
    if (!rc) rc = read_i32(S.inj_d, std::min(ne[sp], S.inj_cap), dst);
    if (rc) return rc;
    std::vector<int64_t> need(ncy);
    for (int j = 0; j < ncy; ++j)
      need[j] = (int64_t)ns[j] + (j > 0 ? nu[j - 1] : 0) + (j + 1 < ncy ? nd[j + 1] : 0);
    for (int32_t d : dst)
      if (d >= 0 && d < ncy) ++need[d];
    rc = fit_rows(c, sp, need, S.nstay);
    if (rc) return rc;
  }
  CU(cudaMemsetAsync(&c->ctl->halt, 0, sizeof(int32_t), c->stream));
  CU(cudaMemsetAsync(&c->ctl->skipped, 0, sizeof(int32_t), c->stream));
  CU(launch_arrive(c->a, c->stream));
  CU(launch_inject_append(c->a, c->stream));
  CU(launch_finalize(c->a, c->stream));
  for (int sp = 0; sp < 2; ++sp) {
    const int rc = fit_staging(c, sp);
    if (rc) return rc;
  }
  int32_t cur = 0;
  CU(cudaStreamSynchronize(c->stream));
  CU(cudaMemcpy(&cur, &c->ctl->cur, sizeof(cur), cudaMemcpyDeviceToHost));
  c->host_cur = cur;
  return launch_steps(c, (int64_t)skipped - 1);
}

// Waits for the context's work; a run that the room check halted is
// completed first, as often as it halts again.  When its rows cannot grow,
// the run stays halted: the context keeps CUPIC_FLAG_CAPACITY and every
// later call that needs its state returns the growth's status, until
// cupic_clear_flags.
int settle(cupic_ctx *c) {
  if (c->grow_status) return c->grow_status;
  for (;;) {
    CU(cudaStreamSynchronize(c->stream));
    int32_t hs[2];
    static_assert(offsetof(Ctl, skipped) == offsetof(Ctl, halt) + 4, "Ctl layout");
    CU(cudaMemcpy(hs, &c->ctl->halt, sizeof(hs), cudaMemcpyDeviceToHost));
    if (!hs[0]) return CUPIC_OK;
    const int rc = complete_halted(c, hs[1]);
    if (rc) {
      c->host_flags |= CUPIC_FLAG_CAPACITY;
      c->grow_status = rc;
      return rc;
    }
  }
}

int get_row_counts(cupic_ctx *c, int sp, std::vector<int32_t> &cnt) {
  cnt.resize(c->p.ncy);
  int rc = settle(c);
  if (rc) return rc;
  CU(cudaMemcpy(cnt.data(), c->a.sp[sp].cnt, c->p.ncy * sizeof(int32_t), cudaMemcpyDeviceToHost));
  return CUPIC_OK;
}

// species sp in row order into host memory, as float4 (out32) or as the
// reference's 4-double struct (out64), with one device-to-host copy
int store_species(cupic_ctx *c, int sp, float *out32, double *out64, int64_t capacity,
                  int64_t *n_out) {
  std::vector<int32_t> cnt;
  int rc = get_row_counts(c, sp, cnt);
  if (rc) return rc;
  const int ncy = c->p.ncy;
  std::vector<int64_t> off(ncy + 1, 0);
  for (int j = 0; j < ncy; ++j) off[j + 1] = off[j] + cnt[j];
  const int64_t n = off[ncy];
  if (n_out) *n_out = n;
  if (n > capacity || (n > 0 && !out32 && !out64)) return CUPIC_ERR_ARG;
  if (n == 0) return CUPIC_OK;
  void *out = out64 ? (void *)out64 : (void *)out32;
  const size_t bytes = (size_t)n * (out64 ? 32 : 16);
  // rows packed into the scratch, then one copy out: on GB300 this copy
  // outruns the packing kernel writing a mapped host array in place
  // (182 vs 79 GB/s for 6.7 GB)
  const size_t b_off = align256((ncy + 1) * sizeof(int64_t));
  void *scratch = nullptr;
  CU(io_scratch(c, b_off + bytes, &scratch));
  int64_t *doff = static_cast<int64_t *>(scratch);
  void *packed = static_cast<unsigned char *>(scratch) + b_off;
  cudaError_t e = cudaMemcpyAsync(doff, off.data(), (ncy + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                                  c->stream);
  if (e == cudaSuccess)
    e = launch_pack_rows(c->a, sp, doff, out64 ? nullptr : (float4 *)packed,
                         out64 ? (double *)packed : nullptr, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, packed, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? CUPIC_OK : cuda_status(e);
}

bool read_line(const char *path, int n, char *line, size_t cap) {
  FILE *f = fopen(path, "r");
  if (!f) return false;
  bool ok = fgets(line, (int)cap, f) != nullptr;
  for (int i = 0; ok && i < n; ++i) ok = fgets(line, (int)cap, f) != nullptr;
  fclose(f);
  return ok;
}

bool read_d(const char *path, int n, double *v) {
  char line[256];
  return read_line(path, n, line, sizeof line) && sscanf(line, "%*s = %lf;", v) == 1;
}

bool read_i(const char *path, int n, int *v) {
  char line[256];
  return read_line(path, n, line, sizeof line) && sscanf(line, "%*s = %d;", v) == 1;
}

}  // namespace

int cupic_ctx_finish(cupic_ctx *c) { return finish(c); }

extern "C" {

const char *cupic_strerror(int s) {
  switch (s) {
    case CUPIC_OK: return "ok";
    case CUPIC_ERR_ARG: return "invalid argument";
    case CUPIC_ERR_CUDA: return "CUDA runtime error";
    case CUPIC_ERR_NOMEM: return "out of memory";
    case CUPIC_ERR_IO: return "input file could not be read";
    case CUPIC_ERR_CAPACITY: return "row or staging capacity exceeded";
    case CUPIC_ERR_CFL: return "a particle moved more than one cell row (or Lx) in one step";
    case CUPIC_ERR_NONFINITE: return "non-finite particle coordinate";
    case CUPIC_ERR_STATE: return "call out of order";
    case CUPIC_ERR_TIMEOUT: return "a bounded device wait gave up";
    case CUPIC_ERR_NODEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

int cupic_params_finalize(cupic_params *p) {
  if (!p) return CUPIC_ERR_ARG;
  const double Lx = p->ds * p->ncx;
  p->ppr = (int32_t)(p->n * Lx * p->ds * p->ds); /* init.cu:136 */
  return CUPIC_OK;
}

int cupic_params_default(cupic_params *p) {
  if (!p) return CUPIC_ERR_ARG;
  memset(p, 0, sizeof(*p));
  p->ncx = 64;
  p->ncy = 256;
  p->ds = 0.5;
  p->dt = 0.05;
  p->n = 160.0;
  p->eps0 = 160.0;
  p->phi_p = -5.0;
  p->me = 1.0;
  p->mi = 100.0;
  p->kte = 1.0;
  p->kti = 1.0;
  p->qe = -1.0;
  p->qi = 1.0;
  p->tol = 1e-6;
  p->min_sweeps = 1;
  p->max_sweeps = 2000;
  p->check_every = 1;
  p->init_tol = 1e-3;
  p->init_min_sweeps = 1;
  p->init_max_sweeps = 2000;
  p->n_save = 100;
  p->n_fin = 1000;
  p->row_slack = 0.5;
  p->stage_frac = 0.25;
  return cupic_params_finalize(p);
}

/* read_input_file + init_* getters (init.cu:424-789): the 13 parameters
 * are lines 1..13 after the header, each "name = value;" */
int cupic_params_from_input_data(const char *path, cupic_params *p) {
  if (!path || !p) return CUPIC_ERR_ARG;
  cupic_params_default(p);
  int n_ini, n_prev, n_save, n_fin, ncx, ncy;
  double ne, Te, beta, gamma, phi_p, ds, dt;
  if (!read_i(path, 1, &n_ini) || !read_i(path, 2, &n_prev) || !read_i(path, 3, &n_save) ||
      !read_i(path, 4, &n_fin) || !read_d(path, 5, &ne) || !read_d(path, 6, &Te) ||
      !read_d(path, 7, &beta) || !read_d(path, 8, &gamma) || !read_d(path, 9, &phi_p) ||
      !read_i(path, 10, &ncx) || !read_i(path, 11, &ncy) || !read_d(path, 12, &ds) ||
      !read_d(path, 13, &dt))
    return CUPIC_ERR_IO;
  const double ME = 9.109e-31, E = 1.602e-19, KB = 1.381e-23, EPS = 8.854e-12; /* init.h:24-27 */
  const double Dl = sqrt(EPS * KB * Te / (ne * E * E));                       /* init.cu:729 */
  double n = ne;
  n *= Dl * Dl * Dl; /* init.cu:552 */
  double eps = EPS;  /* init.cu:622-626 */
  eps /= pow(Dl * sqrt(ME / (KB * Te)), 2);
  eps /= E * E;
  eps *= Dl * Dl * Dl;
  eps *= ME;
  double php = phi_p;
  php *= E / (KB * Te); /* init.cu:534 */
  p->n_ini = n_ini;
  p->n_prev = n_prev;
  p->n_save = n_save;
  p->n_fin = n_fin;
  p->ncx = ncx;
  p->ncy = ncy;
  p->ds = ds;
  p->dt = dt;
  p->n = n;
  p->eps0 = eps;
  p->phi_p = php;
  p->mi = gamma;
  p->kti = beta;
  const int mn = std::max(ncx + 1, ncy + 1) + 1; /* mesh.cu:67,94: sweeps >= max(nnx,nny)+1 */
  p->tol = 1e-4;                                 /* main.cu:64 */
  p->min_sweeps = mn;
  p->max_sweeps = 1000000;
  p->check_every = 1;
  p->init_tol = 1e-3; /* init.cu:254 */
  p->init_min_sweeps = mn;
  p->init_max_sweeps = 1000000;
  return cupic_params_finalize(p);
}

int cupic_create(const cupic_params *pin, int device, cupic_ctx **out) {
  if (!out) return CUPIC_ERR_ARG;
  *out = nullptr;
  int rc = validate(pin);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return CUPIC_ERR_NODEVICE;
  }
  if (device < 0 || device >= ndev) return CUPIC_ERR_ARG;
  cupic_ctx *c = new (std::nothrow) cupic_ctx();
  if (!c) return CUPIC_ERR_NOMEM;
  c->p = *pin;
  c->device = device;
  auto fail = [&](int r) {
    cupic_destroy(c);
    return r;
  };
  if (cudaSetDevice(device) != cudaSuccess) return fail(CUPIC_ERR_CUDA);
  if (cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      keep_pool(device) != cudaSuccess)
    return fail(CUPIC_ERR_CUDA);
  {
    StreamSet s{};
    const cudaError_t e = take_stream_set(device, &s);
    c->stream = s.stream;
    c->side = s.side;
    c->ev_fork = s.fork;
    c->ev_join = s.join;
    if (e != cudaSuccess) return fail(CUPIC_ERR_CUDA);
  }
  fill_constants(c);
  SimArgs &a = c->a;
  const size_t nodes = (size_t)a.nnx * a.nny;
  if (dalloc(c, &a.phi, nodes) || dalloc(c, &a.E, nodes) || dalloc(c, &a.rho[0], nodes) ||
      dalloc(c, &a.rho[1], nodes) || dalloc(c, &c->ctl, 1))
    return fail(CUPIC_ERR_NOMEM);
  a.ctl = c->ctl;
  if (c->p.refine_every > 0) {
    if (dalloc(c, &c->phi64, nodes) || dalloc(c, &c->b64, nodes) || dalloc(c, &c->rr, nodes) || dalloc(c, &c->dl, nodes) ||
        dalloc(c, &c->maxr, 1) || cudaMallocHost(&c->h_pin, 64) != cudaSuccess)
      return fail(CUPIC_ERR_NOMEM);
    if (cudaMemsetAsync(c->phi64, 0, nodes * sizeof(double), c->stream)) return fail(CUPIC_ERR_CUDA);
  }
  // set-up is ordered on the context's stream: creating a context never
  // waits for the device, which may be busy with other contexts' steps
  if (cudaMemsetAsync(a.phi, 0, nodes * sizeof(float), c->stream) ||
      cudaMemsetAsync(a.E, 0, nodes * sizeof(float2), c->stream) ||
      cudaMemsetAsync(a.rho[0], 0, nodes * 8, c->stream) ||
      cudaMemsetAsync(a.rho[1], 0, nodes * 8, c->stream) ||
      cudaMemsetAsync(c->ctl, 0, sizeof(Ctl), c->stream))
    return fail(CUPIC_ERR_CUDA);
  const int32_t capj = round8(c->p.ppr * (1.0 + c->p.row_slack)) + 64;
  for (int sp = 0; sp < 2; ++sp) {
    const double per_step = c->p.dt / a.dtin[sp];
    a.sp[sp].inj_cap = (int32_t)std::min(4.0 * ceil(per_step) + 1024.0, 1.0e8);
    rc = layout_species(c, sp, std::vector<int32_t>(c->p.ncy, capj));
    if (rc) return fail(rc);
  }
  rc = plan_jacobi(c);
  if (rc) return fail(rc);
  if (push_set_smem(push_smem_bytes(a.nnx)) != cudaSuccess) return fail(CUPIC_ERR_ARG);
  rc = cupic_set_time(c, (int64_t)c->p.n_ini + 1, c->p.n_ini * c->p.dt + c->p.dt, -1.0, -1.0);
  if (rc) return fail(rc);
  *out = c;
  return CUPIC_OK;
}

int cupic_destroy(cupic_ctx *c) {
  if (!c) return CUPIC_ERR_ARG;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->side) cudaStreamSynchronize(c->side);
  destroy_graph(c);
  // stream-ordered frees on the context's stream, which the streams'
  // destruction below lets finish
  for (int sp = 0; sp < 2; ++sp) free_species(c, c->a.sp[sp]);
  dfree(c, c->a.phi);
  dfree(c, c->a.E);
  dfree(c, c->a.rho[0]);
  dfree(c, c->a.rho[1]);
  dfree(c, c->ctl);
  dfree(c, c->jflags);
  dfree(c, c->jres);
  dfree(c, c->jhalo);
  dfree(c, c->io_buf);
  dfree(c, c->phi64);
  dfree(c, c->b64);
  dfree(c, c->rr);
  dfree(c, c->dl);
  dfree(c, c->maxr);
  if (c->h_pin) cudaFreeHost(c->h_pin);
  if (c->stream && c->side && c->ev_fork && c->ev_join) {
    // back to the device's set for the next context (the frees above run
    // on the stream, before any later work the next owner enqueues)
    keep_stream_set(c->device, {c->stream, c->side, c->ev_fork, c->ev_join});
  } else {
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->stream) cudaStreamDestroy(c->stream);
  }
  delete c;
  return CUPIC_OK;
}

int cupic_set_time(cupic_ctx *c, int64_t step, double t, double tin_e, double tin_i) {
  if (!c) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  // ordered on the context's stream after the work already enqueued there
  CU(launch_set_time(c->ctl, step, t, tin_e, tin_i, c->stream));
  return CUPIC_OK;
}

int cupic_get_time(cupic_ctx *c, int64_t *step, double *t, double *tin_e, double *tin_i) {
  if (!c) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  SETTLE(c);
  struct {
    int64_t step;
    double t;
    double tin[2];
    int32_t tin_set[2];
  } h;
  CU(cudaMemcpy(&h, c->ctl, sizeof(h), cudaMemcpyDeviceToHost));
  if (step) *step = h.step;
  if (t) *t = h.t;
  if (tin_e) *tin_e = h.tin_set[0] ? h.tin[0] : -1.0;
  if (tin_i) *tin_i = h.tin_set[1] ? h.tin[1] : -1.0;
  return CUPIC_OK;
}

// init_sim's n_ini == 0 branch (init.cu:70-83), enqueued on the context's
// stream without waiting for it
int init_plasma_enqueue(cupic_ctx *c) {
  CU(cudaSetDevice(c->device));
  const int capj = c->cap[0].empty() ? 0 : *std::min_element(c->cap[0].begin(), c->cap[0].end());
  if (capj < c->p.ppr) return CUPIC_ERR_CAPACITY;
  // a halted run that was never completed is discarded with the old state
  static_assert(offsetof(Ctl, skipped) == offsetof(Ctl, halt) + 4, "Ctl layout");
  CU(cudaMemsetAsync(&c->ctl->halt, 0, 2 * sizeof(int32_t), c->stream));
  CU(launch_init_particles(c->a, c->stream));
  int rc = set_linear_phi(c);
  if (rc) return rc;
  rc = deposit_current(c);
  if (rc) return rc;
  const cupic_params &p = c->p;
  rc = epoch_guard(c, solves_of(c, p.init_max_sweeps));
  if (!rc) rc = run_solve(c, p.init_tol, p.init_min_sweeps, p.init_max_sweeps, p.check_every, 1);
  if (rc) return rc;
  CU(launch_leapfrog_start(c->a, c->stream));
  rc = cupic_set_time(c, (int64_t)p.n_ini + 1, p.n_ini * p.dt + p.dt, -1.0, -1.0);
  if (rc) return rc;
  c->initialized = true;
  return CUPIC_OK;
}

int cupic_init_plasma(cupic_ctx *c) {
  if (!c) return CUPIC_ERR_ARG;
  const int rc = init_plasma_enqueue(c);
  return rc ? rc : finish(c);
}

int cupic_reserve(int device, uint64_t bytes, int32_t contexts) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev || contexts < 0) {
    cudaGetLastError();
    return CUPIC_ERR_ARG;
  }
  CU(cudaSetDevice(device));
  CU(keep_pool(device));
  int have = 0;
  {
    std::lock_guard<std::mutex> lk(g_streams_mu);
    if ((int)g_streams.size() > device) have = (int)g_streams[device].size();
  }
  for (int k = have; k < contexts; ++k) {
    StreamSet s{};
    CU(new_stream_set(&s));
    keep_stream_set(device, s);
  }
  if (bytes == 0) return CUPIC_OK;
  // Grow the pool only when the memory it already holds and does not use
  // falls short.  A pool that earlier contexts have left holding freed
  // memory in many pieces must not be grown past it: after such a growth
  // every context created while the device is busy waited for the device
  // (52 ms each in a serving run after 512 contexts had come and gone,
  // against 0.05 ms without the growth).
  {
    cudaMemPool_t pool;
    CU(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t reserved = 0, used = 0;
    CU(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved));
    CU(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used));
    if (reserved >= used && reserved - used >= bytes) return CUPIC_OK;
  }
  cudaStream_t st = nullptr;
  CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  void *p = nullptr;
  cudaError_t e = cudaMallocAsync(&p, (size_t)bytes, st);
  if (e == cudaSuccess) e = cudaFreeAsync(p, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  return e == cudaSuccess ? CUPIC_OK : cuda_status(e);
}

int cupic_init_plasma_nowait(cupic_ctx *c) {
  if (!c) return CUPIC_ERR_ARG;
  return init_plasma_enqueue(c);
}

int cupic_init_mesh(cupic_ctx *c) {
  if (!c) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  CU(cudaStreamSynchronize(c->stream));
  int rc = set_linear_phi(c);
  if (rc) return rc;
  rc = deposit_current(c);
  if (rc) return rc;
  const cupic_params &p = c->p;
  rc = epoch_guard(c, solves_of(c, p.init_max_sweeps));
  if (!rc) rc = run_solve(c, p.init_tol, p.init_min_sweeps, p.init_max_sweeps, p.check_every, 1);
  if (rc) return rc;
  rc = sync_check(c);
  if (rc) return rc;
  rc = cupic_set_time(c, (int64_t)p.n_ini + 1, p.n_ini * p.dt + p.dt, -1.0, -1.0);
  if (rc) return rc;
  c->initialized = true;
  return finish(c);
}

int cupic_get_params(cupic_ctx *c, cupic_params *p) {
  if (!c || !p) return CUPIC_ERR_ARG;
  *p = c->p;
  return CUPIC_OK;
}

int cupic_get_solver_plan(cupic_ctx *c, int32_t *ctas, int32_t *rows_per_cta, int32_t *depth) {
  if (!c) return CUPIC_ERR_ARG;
  if (ctas) *ctas = c->jG;
  if (rows_per_cta) *rows_per_cta = c->jB;
  if (depth) *depth = c->jK;
  return CUPIC_OK;
}

int cupic_load_particles(cupic_ctx *c, int sp, const double *xyvv, int64_t n) {
  if (!c || sp < 0 || sp > 1 || n < 0 || (n > 0 && !xyvv)) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  SETTLE(c);
  const int ncy = c->p.ncy;
  const int nb = load_blocks(n, c->num_sms);
  // a mapped host array is read in place by the conversion kernel (as fast
  // as a copy, and no staging memory); a pageable one is first copied into
  // the scratch
  const double *mapped = n > 0 ? static_cast<const double *>(mapped_host(xyvv)) : nullptr;
  const size_t b_tmp = align256((size_t)n * sizeof(float4));
  const size_t b_h = align256((size_t)nb * ncy * sizeof(int32_t));
  const size_t b_in = mapped ? 0 : align256((size_t)n * 32);
  // sized for a download of as many particles too, so that the download
  // that usually follows does not grow it again
  const size_t b_down = align256((ncy + 1) * sizeof(int64_t)) + (size_t)n * 32;
  void *scratch = nullptr;
  CU(io_scratch(c, std::max(b_tmp + b_h + 256 + b_in, b_down), &scratch));
  unsigned char *q = static_cast<unsigned char *>(scratch);
  float4 *tmp = reinterpret_cast<float4 *>(q);
  int32_t *H = reinterpret_cast<int32_t *>(q + b_tmp);
  unsigned *bad = reinterpret_cast<unsigned *>(q + b_tmp + b_h);
  const double *din = mapped ? mapped : reinterpret_cast<const double *>(q + b_tmp + b_h + 256);
  std::vector<int32_t> cnt(ncy, 0);
  unsigned hbad = 0;
  int rc = CUPIC_OK;
  cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(unsigned), c->stream);
  if (e == cudaSuccess && n > 0 && !mapped)
    e = cudaMemcpyAsync(const_cast<double *>(din), xyvv, (size_t)n * 32, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && n > 0) e = launch_load_hist(c->a, din, n, nb, tmp, H, bad, c->stream);
  if (e == cudaSuccess && n > 0) e = launch_load_scan(H, nb, ncy, c->a.sp[sp].cnt, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hbad, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess && n > 0)
    e = cudaMemcpyAsync(cnt.data(), c->a.sp[sp].cnt, ncy * sizeof(int32_t), cudaMemcpyDeviceToHost,
                        c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) rc = cuda_status(e);
  if (!rc && hbad) rc = CUPIC_ERR_ARG;
  if (!rc) {
    bool grow = false;
    std::vector<int32_t> capv = c->cap[sp];
    for (int j = 0; j < ncy; ++j)
      if (cnt[j] > capv[j]) {
        capv[j] = round8(cnt[j] * (1.0 + c->p.row_slack)) + 64;
        grow = true;
      }
    if (grow) rc = layout_species(c, sp, capv);
    if (!rc) {
      e = cudaMemcpyAsync(c->a.sp[sp].cnt, cnt.data(), ncy * sizeof(int32_t),
                          cudaMemcpyHostToDevice, c->stream);
      if (e == cudaSuccess && n > 0) e = launch_load_scatter(c->a, sp, tmp, n, nb, H, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) rc = cuda_status(e);
    }
  }
  if (rc) return rc;
  c->rho_valid = false;
  c->initialized = true;
  return CUPIC_OK;
}

int cupic_charge_deposition(cupic_ctx *c) {
  if (!c) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  // a step's push already deposited the moved and injected particles into
  // the accumulator the next solve reads; the integer sums are identical
  if (c->rho_valid) return sync_check(c);
  int rc = deposit_current(c);
  if (rc) return rc;
  return sync_check(c);
}

int cupic_poisson_solver(cupic_ctx *c, double max_error, int32_t mn, int32_t mx, int32_t chk) {
  if (!c) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  if (!c->rho_valid) {
    int rc = deposit_current(c);
    if (rc) return rc;
  }
  if (max_error < 0) {
    max_error = c->p.tol;
    mn = c->p.min_sweeps;
    mx = c->p.max_sweeps;
    chk = c->p.check_every;
  }
  if (mx < 0) return CUPIC_ERR_ARG;
  int rc = epoch_guard(c, solves_of(c, mx));
  if (!rc) rc = run_solve(c, max_error, mn, mx, chk, 0);
  if (rc) return rc;
  return finish(c);
}

int cupic_field_solver(cupic_ctx *c) {
  if (!c) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  if (c->p.refine_every > 0) {
    CU(launch_r64_field(c->a, c->phi64, c->stream));
  } else {
    JacobiArgs J = jargs(c, 0.0, 0, 0, 1, 1);
    J.write_stats = 0;
    int rc = epoch_guard(c, 1);
    if (rc) return rc;
    CU(launch_jacobi(c->a, J, c->stream));
  }
  return finish(c);
}

int cupic_particle_mover(cupic_ctx *c) {
  if (!c) return CUPIC_ERR_ARG;
  if (!c->initialized) return CUPIC_ERR_STATE;
  CU(cudaSetDevice(c->device));
  CU(launch_zero_next_rho(c->a, c->stream));
  CU(launch_push_deposit(c->a, c->stream));
  // rows that cannot take their stayers and the movers staged for them
  // grow first (the step's graph does this with the room check)
  CU(cudaStreamSynchronize(c->stream));
  const int ncy = c->p.ncy;
  for (int sp = 0; sp < 2; ++sp) {
    const SpeciesDev &S = c->a.sp[sp];
    std::vector<int32_t> ns, nu, nd;
    int rc = read_i32(S.nstay, ncy, ns);
    if (!rc) rc = read_i32(S.nup, ncy, nu);
    if (!rc) rc = read_i32(S.ndown, ncy, nd);
    if (rc) return rc;
    std::vector<int64_t> need(ncy);
    for (int j = 0; j < ncy; ++j)
      need[j] = (int64_t)ns[j] + (j > 0 ? nu[j - 1] : 0) + (j + 1 < ncy ? nd[j + 1] : 0);
    rc = fit_rows(c, sp, need, S.nstay);
    if (rc) return rc;
  }
  CU(launch_arrive(c->a, c->stream));
  for (int sp = 0; sp < 2; ++sp) {
    const int rc = fit_staging(c, sp);
    if (rc) return rc;
  }
  c->rho_valid = false;  // until cc completes the next charge
  return finish(c);
}

int cupic_cc(cupic_ctx *c, double t) {
  if (!c) return CUPIC_ERR_ARG;
  if (!c->initialized) return CUPIC_ERR_STATE;
  CU(cudaSetDevice(c->device));
  SETTLE(c);
  CU(cudaMemcpy(&c->ctl->t, &t, sizeof(double), cudaMemcpyHostToDevice));
  CU(launch_inject_draw(c->a, c->stream));
  // rows that cannot take the injected particles grow first
  CU(cudaStreamSynchronize(c->stream));
  const int ncy = c->p.ncy;
  int32_t ne[2] = {0, 0};
  CU(cudaMemcpy(ne, c->ctl->inj_gen, sizeof(ne), cudaMemcpyDeviceToHost));
  for (int sp = 0; sp < 2; ++sp) {
    const SpeciesDev &S = c->a.sp[sp];
    std::vector<int32_t> cnt, dst;
    int rc = read_i32(S.cnt, ncy, cnt);
    if (!rc) rc = read_i32(S.inj_d, std::min(ne[sp], S.inj_cap), dst);
    if (rc) return rc;
    std::vector<int64_t> need(cnt.begin(), cnt.end());
    for (int32_t d : dst)
      if (d >= 0 && d < ncy) ++need[d];
    rc = fit_rows(c, sp, need, S.cnt);
    if (rc) return rc;
  }
  CU(launch_inject_append(c->a, c->stream));
  CU(launch_finalize(c->a, c->stream));
  c->host_cur ^= 1;
  c->rho_valid = true;
  return finish(c);
}

int cupic_step(cupic_ctx *c, int32_t nsteps) {
  if (!c || nsteps < 0) return CUPIC_ERR_ARG;
  if (!c->initialized) return CUPIC_ERR_STATE;
  CU(cudaSetDevice(c->device));
  if (!c->rho_valid) {
    int rc = deposit_current(c);
    if (rc) return rc;
  }
  if (c->p.refine_every > 0 && !refine_on_device(c, c->p.max_sweeps)) {
    // the solve reads its residual norm on the host: no graph, and a step
    // that runs out of room is completed before the next one starts
    for (int i = 0; i < nsteps; ++i) {
      int rc = epoch_guard(c, solves_of(c, c->p.max_sweeps));
      if (!rc) rc = enqueue_step(c);
      if (!rc) c->host_cur ^= 1;
      if (!rc) rc = settle(c);
      if (rc) return rc;
    }
    return CUPIC_OK;
  }
  return launch_steps(c, nsteps);
}

int cupic_sync(cupic_ctx *c) {
  if (!c) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  return finish(c);
}

int cupic_get_counts(cupic_ctx *c, int64_t *ne, int64_t *ni) {
  if (!c) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  for (int sp = 0; sp < 2; ++sp) {
    std::vector<int32_t> cnt;
    int rc = get_row_counts(c, sp, cnt);
    if (rc) return rc;
    int64_t s = 0;
    for (int32_t v : cnt) s += v;
    if (sp == 0 && ne) *ne = s;
    if (sp == 1 && ni) *ni = s;
  }
  return CUPIC_OK;
}

int cupic_store_particles_f32(cupic_ctx *c, int sp, float *out, int64_t capacity, int64_t *n_out) {
  if (!c || sp < 0 || sp > 1) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  return store_species(c, sp, out, nullptr, capacity, n_out);
}

int cupic_store_particles(cupic_ctx *c, int sp, double *out, int64_t capacity, int64_t *n_out) {
  if (!c || sp < 0 || sp > 1) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  if (!out) {
    std::vector<int32_t> cnt;
    int rc = get_row_counts(c, sp, cnt);
    if (rc) return rc;
    int64_t n = 0;
    for (int32_t v : cnt) n += v;
    if (n_out) *n_out = n;
    return n == 0 ? CUPIC_OK : CUPIC_ERR_ARG;
  }
  return store_species(c, sp, nullptr, out, capacity, n_out);
}

int cupic_step_timed(cupic_ctx *c, int32_t nsteps, float *phase_ms, int32_t nphase,
                     float *total_ms) {
  if (!c || nsteps < 1 || !phase_ms || nphase < CUPIC_NPHASE || !total_ms) return CUPIC_ERR_ARG;
  if (!c->initialized) return CUPIC_ERR_STATE;
  CU(cudaSetDevice(c->device));
  if (!c->rho_valid) {
    int rc = deposit_current(c);
    if (rc) return rc;
  }
  // the step's own launch sequence (enqueue_step, the one its graph
  // captures), launched directly with an event after each phase
  const int per = CUPIC_NPHASE;
  std::vector<cudaEvent_t> ev((size_t)nsteps * per + 2, nullptr);
  int rc = CUPIC_OK;
  for (auto &e : ev)
    if (cudaEventCreate(&e) != cudaSuccess) rc = CUPIC_ERR_CUDA;
  cudaError_t e = rc ? cudaErrorUnknown : cudaEventRecord(ev[0], c->stream);
  for (int s = 0; s < nsteps && e == cudaSuccess && !rc; ++s) {
    rc = epoch_guard(c, solves_of(c, c->p.max_sweeps));
    if (!rc) rc = enqueue_step(c, &ev[(size_t)s * per + 1]);
    if (!rc) c->host_cur ^= 1;
  }
  if (e == cudaSuccess && !rc) e = cudaStreamSynchronize(c->stream);
  // a run halted by the room check is completed (rows grown, the halted
  // step finished, the skipped steps run) inside the timed region
  int32_t halted = 0;
  if (e == cudaSuccess && !rc) e = cudaMemcpy(&halted, &c->ctl->halt, sizeof(halted), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && !rc && halted) {
    rc = settle(c);
    if (!rc) e = cudaEventRecord(ev.back(), c->stream);
    if (e == cudaSuccess && !rc) e = cudaStreamSynchronize(c->stream);
  }
  for (int k = 0; k < nphase; ++k) phase_ms[k] = 0.0f;
  if (e == cudaSuccess && !rc) {
    for (int s = 0; s < nsteps && e == cudaSuccess; ++s)
      for (int k = 0; k < per && e == cudaSuccess; ++k) {
        float ms = 0.0f;
        e = cudaEventElapsedTime(&ms, ev[(size_t)s * per + k], ev[(size_t)s * per + k + 1]);
        phase_ms[k] += ms;
      }
    if (e == cudaSuccess) e = cudaEventElapsedTime(total_ms, ev[0], halted ? ev.back() : ev[ev.size() - 2]);
  }
  for (auto &x : ev)
    if (x) cudaEventDestroy(x);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_status(e);
  return finish(c);
}

int cupic_get_bookmarks(cupic_ctx *c, int sp, int32_t *bm) {
  if (!c || sp < 0 || sp > 1 || !bm) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  std::vector<int32_t> cnt;
  int rc = get_row_counts(c, sp, cnt);
  if (rc) return rc;
  int64_t off = 0;
  for (int j = 0; j < c->p.ncy; ++j) {
    if (cnt[j] > 0) {
      bm[2 * j] = (int32_t)off;
      bm[2 * j + 1] = (int32_t)(off + cnt[j] - 1);
    } else {
      bm[2 * j] = bm[2 * j + 1] = -1;
    }
    off += cnt[j];
  }
  return CUPIC_OK;
}

int cupic_get_rho_fixed(cupic_ctx *c, int which, int64_t *acc) {
  if (!c || !acc || which < 0 || which > 1) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  if (which == 0 && !c->rho_valid) {
    int rc = deposit_current(c);
    if (rc) return rc;
  }
  SETTLE(c);
  const size_t nodes = (size_t)c->a.nnx * c->a.nny;
  CU(cudaMemcpy(acc, c->a.rho[c->host_cur ^ which], nodes * sizeof(int64_t), cudaMemcpyDeviceToHost));
  return CUPIC_OK;
}

int cupic_get_rho(cupic_ctx *c, int which, double *rho) {
  if (!c || !rho) return CUPIC_ERR_ARG;
  const int nnx = c->a.nnx, nny = c->a.nny;
  std::vector<int64_t> acc((size_t)nnx * nny);
  int rc = cupic_get_rho_fixed(c, which, acc.data());
  if (rc) return rc;
  const double ds3 = c->p.ds * c->p.ds * c->p.ds, scale = ldexp(1.0, -32);
  for (int j = 0; j < nny; ++j) {
    const double vol = (j == 0 || j == nny - 1) ? 0.5 * ds3 : ds3;
    const size_t r = (size_t)j * nnx;
    for (int i = 0; i < nnx; ++i) {
      const int64_t f = (i == 0 || i == nnx - 1) ? acc[r] + acc[r + nnx - 1] : acc[r + i];
      rho[r + i] = (double)f * scale / vol;
    }
  }
  return CUPIC_OK;
}

int cupic_get_phi_f32(cupic_ctx *c, float *phi) {
  if (!c || !phi) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  SETTLE(c);
  CU(cudaMemcpy(phi, c->a.phi, sizeof(float) * (size_t)c->a.nnx * c->a.nny, cudaMemcpyDeviceToHost));
  return CUPIC_OK;
}

int cupic_get_phi(cupic_ctx *c, double *phi) {
  if (!c || !phi) return CUPIC_ERR_ARG;
  if (c->phi64) {  // the precision form's FP64 potential
    CU(cudaSetDevice(c->device));
    SETTLE(c);
    CU(cudaMemcpy(phi, c->phi64, sizeof(double) * c->a.nnx * c->a.nny, cudaMemcpyDeviceToHost));
    return CUPIC_OK;
  }
  std::vector<float> h((size_t)c->a.nnx * c->a.nny);
  int rc = cupic_get_phi_f32(c, h.data());
  if (rc) return rc;
  for (size_t k = 0; k < h.size(); ++k) phi[k] = (double)h[k];
  return CUPIC_OK;
}

int cupic_set_phi(cupic_ctx *c, const double *phi) {
  if (!c || !phi) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  SETTLE(c);
  return set_phi_both(c, phi);
}

int cupic_get_field_f32(cupic_ctx *c, float *ex, float *ey) {
  if (!c || !ex || !ey) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  SETTLE(c);
  const size_t nodes = (size_t)c->a.nnx * c->a.nny;
  std::vector<float2> h(nodes);
  CU(cudaMemcpy(h.data(), c->a.E, nodes * sizeof(float2), cudaMemcpyDeviceToHost));
  for (size_t k = 0; k < nodes; ++k) {
    ex[k] = h[k].x;
    ey[k] = h[k].y;
  }
  return CUPIC_OK;
}

int cupic_get_field(cupic_ctx *c, double *ex, double *ey) {
  if (!c || !ex || !ey) return CUPIC_ERR_ARG;
  const size_t nodes = (size_t)c->a.nnx * c->a.nny;
  std::vector<float> hx(nodes), hy(nodes);
  int rc = cupic_get_field_f32(c, hx.data(), hy.data());
  if (rc) return rc;
  for (size_t k = 0; k < nodes; ++k) {
    ex[k] = hx[k];
    ey[k] = hy[k];
  }
  return CUPIC_OK;
}

int cupic_get_stats(cupic_ctx *c, cupic_step_stats *out, int32_t count) {
  if (!c || !out || count < 0 || count > kStatsRing) return CUPIC_ERR_ARG;
  if (count == 0) return CUPIC_OK;
  CU(cudaSetDevice(c->device));
  SETTLE(c);
  int64_t step = 0;
  CU(cudaMemcpy(&step, &c->ctl->step, sizeof(step), cudaMemcpyDeviceToHost));
  // the ring entries of steps step-count .. step-1, in at most two copies
  const int64_t first = (((step - count) % kStatsRing) + kStatsRing) % kStatsRing;
  const int64_t n1 = std::min<int64_t>(count, kStatsRing - first);
  CU(cudaMemcpy(out, &c->ctl->ring[first], n1 * sizeof(cupic_step_stats), cudaMemcpyDeviceToHost));
  if (n1 < count)
    CU(cudaMemcpy(out + n1, &c->ctl->ring[0], (count - n1) * sizeof(cupic_step_stats),
                  cudaMemcpyDeviceToHost));
  return CUPIC_OK;
}

int cupic_probe_current(cupic_ctx *c, int32_t window, double *current) {
  if (!c || !current || window < 1 || window > kStatsRing) return CUPIC_ERR_ARG;
  std::vector<cupic_step_stats> st(window);
  int rc = cupic_get_stats(c, st.data(), window);
  if (rc) return rc;
  double sum = 0.0;
  for (const cupic_step_stats &x : st)
    sum += c->p.qe * (double)x.absorbed[0] + c->p.qi * (double)x.absorbed[1];
  *current = sum / window;
  return CUPIC_OK;
}

int cupic_density_profile(cupic_ctx *c, int species, double *density) {
  if (!c || !density || species < 0 || species > 1) return CUPIC_ERR_ARG;
  std::vector<int32_t> cnt;
  int rc = get_row_counts(c, species, cnt);
  if (rc) return rc;
  const double cell = c->p.ds * c->p.ds * c->p.ds;
  for (int j = 0; j < c->p.ncy; ++j) density[j] = cnt[j] / (c->p.ncx * cell);
  return CUPIC_OK;
}

int cupic_get_flags(cupic_ctx *c, uint32_t *flags) {
  if (!c || !flags) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  const int rc = settle(c);
  if (rc && !c->grow_status) return rc;  // a failed growth is reported as a flag
  return read_ctl_flags(c, flags);
}

int cupic_test_bounded_wait(cupic_ctx *c) {
  if (!c) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  CU(launch_wait_probe(c->a, c->stream));
  return finish(c);
}

int cupic_clear_flags(cupic_ctx *c) {
  if (!c) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(c->device));
  // a run whose rows could not grow is retried by the next call
  c->host_flags = 0;
  c->grow_status = 0;
  SETTLE(c);
  uint32_t z[2] = {0u, 0u};
  int32_t zero = 0;
  CU(cudaMemcpy(&c->ctl->flags, z, sizeof(z), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(&c->ctl->abort, &zero, sizeof(zero), cudaMemcpyHostToDevice));
  return CUPIC_OK;
}

}  // extern "C"
