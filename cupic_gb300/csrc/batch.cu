// batch.cu -- many independent contexts (probe-bias instances of uneven
// sizes) stepped together.  It has no counterpart in the reference, which
// runs one simulation per process.
//
// One batched step is one launch per kernel for all members:
//   - the solves: one cooperative launch whose CTAs are split into groups;
//     a group of G CTAs solves its list of instances one after another
//     (instances that fit one CTA's shared memory get G = 1, larger ones the
//     fewest CTAs that hold them, or with few members up to their share of
//     the CTAs), groups sized and filled by the members' mesh work (largest
//     first onto the least-loaded group);
//   - push, arrive and the charge clear: work lists of {instance, row};
//     instances of 512 rows or more, which fill the GPU by themselves, are
//     pushed by the single-context kernel on parallel graph branches;
//   - the injection draws (beside the push, on a side stream), the room
//     check, the append and the bookkeeping: one block or thread per
//     instance and species.
// Every kernel reads its instance's SimArgs from a device array, so members
// keep their own buffers and control blocks, and a member's results are the
// ones it gets when stepped alone.  The step is captured once per
// membership as a CUDA graph.  A member whose rows run out of room halts
// alone (its kernels return at once); the batch's sync grows its rows and
// completes its steps with the single-context step, and the next batched
// step rebuilds the arrays.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <new>
#include <numeric>
#include <tuple>
#include <vector>

#include "ctx.h"
#include "kernels.h"

using namespace cupic;

struct cupic_batch {
  int device = 0, num_sms = 0;
  cudaStream_t stream = nullptr, side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  std::vector<cupic_ctx *> members;
  std::vector<int> epochs;  // members' layout epochs when the arrays were built
  // device arrays, grown as needed
  SimArgs *d_inst = nullptr;
  JacobiArgs *d_jargs = nullptr;
  JGroup *d_groups = nullptr;
  int *d_list = nullptr;
  int2 *d_rows = nullptr;
  unsigned *d_flags = nullptr;
  float *d_res = nullptr;
  unsigned long long *d_halo = nullptr;  // halo words of all solves, zeroed at every build
  size_t cap_inst = 0, cap_groups = 0, cap_rows = 0, cap_flags = 0, cap_res = 0,
         cap_halo = 0;
  int ngroups = 0, nctas = 0, nrows = 0, max_nnx = 0, max_ncy = 0, max_inj = 0;
  // d_rows: rows of short-row instances (ncx <= kShortRow, pushed by
  // 128-thread blocks), then rows of mid-size ones (512-thread blocks),
  // then rows of big ones (ncy >= kBigRows), which are pushed by the
  // single-context kernel, one launch per instance on parallel branches
  int nrows_short = 0, nrows_mid = 0, max_nnx_short = 0, max_nnx_mid = 0;
  std::vector<int> big;  // member indices pushed one launch each
  cudaStream_t push_st[4] = {};
  cudaEvent_t ev_push_fork = nullptr, ev_push_join[4] = {};
  size_t nflags = 0, jsmem = 0;
  cudaGraphExec_t graph = nullptr;
  bool graph_ok = false;
  // the batched solve's layout knobs in use: halo depth cap, CTA multiple;
  // tuned_n: the member count they were tuned for (0: not tuned)
  int knob_depth = 4, knob_mult = 1, tuned_n = 0;
  // batched steps since d_halo was last zeroed: a halo word's epoch holds
  // the solve count in 16 bits, so the words are zeroed before it can wrap
  int64_t epoch_steps = 0;
  size_t nhalo = 0;
};

namespace {

constexpr int kShortRow = 64;  // cells per row up to which 128-thread blocks push a row
constexpr int kBigRows = 512;  // rows from which an instance fills the GPU by itself
constexpr int kPushBranches = 4;

#define CU(call)                                                            \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) return e_ == cudaErrorMemoryAllocation ? CUPIC_ERR_NOMEM \
                                                                  : CUPIC_ERR_CUDA; \
  } while (0)

template <class T>
int grow(T **p, size_t *cap, size_t n) {
  if (n <= *cap && *p) return CUPIC_OK;
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  const size_t m = std::max<size_t>(n, 1);
  CU(cudaMalloc((void **)p, m * sizeof(T)));
  *cap = m;
  return CUPIC_OK;
}

void drop_graph(cupic_batch *b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->graph_ok = false;
}

// The batched solve's layout of one instance: the fewest CTAs whose shared
// memory holds its rows (tile height B = ceil(rows / G)), times a CTA
// multiple, with a halo depth of up to a cap.  The depth cap and the
// multiple are the two knobs of the batched-solve autotuner (tune_solve);
// without tuning they are 4 and 1 (over the 256-instance mix, depths of 2,
// 3, 4, 6, 8 and 16 gave 15.1, 14.6, 14.4, 14.8, 14.6 and 16.1 ms per
// batched step).
struct Knobs {
  int depth, mult;
  bool operator<(const Knobs &o) const { return depth != o.depth ? depth < o.depth : mult < o.mult; }
};
constexpr Knobs kDefaultKnobs{4, 1};
constexpr Knobs kCandidates[] = {{1, 1}, {2, 1}, {4, 1}, {8, 1}, {2, 2}, {4, 2}, {8, 2}};
constexpr int kTuneMembers = 16;  // batches this large tune their solve layout
struct Plan {
  int G, B, K, P;
  size_t smem;
};

// the layout on G > 1 CTAs, if their shared memory holds it
bool plan_on(const SimArgs &a, int G, long long rows_fit, int kcap, Plan *out) {
  const int M = a.nny - 2;
  const int P = (a.nnx + 3) / 4 * 4;
  const int B = (M + G - 1) / G;
  const int K = std::min(kcap, M / G);
  if (G < 2 || K < 1 || B + 2 * K > rows_fit) return false;
  *out = {G, B, K, P, jacobi_smem_bytes(B, K, P)};
  return true;
}

bool plan_instance(const SimArgs &a, long long rows_fit, const Knobs &k, Plan *out) {
  const int M = a.nny - 2;
  const int P = (a.nnx + 3) / 4 * 4;
  Plan base{};
  bool ok = false;
  if (M + 2 <= rows_fit) {
    base = {1, M, 1, P, jacobi_smem_bytes(M, 1, P)};
    ok = true;
  }
  for (int G = 2; !ok && G <= M; ++G) ok = plan_on(a, G, rows_fit, k.depth, &base);
  if (!ok) return false;
  Plan q;
  if (k.mult > 1 && plan_on(a, std::min(M, base.G * k.mult), rows_fit, k.depth, &q)) base = q;
  *out = base;
  return true;
}

// The solve's part of the batch arrays for the given knobs: every member's
// plan, the CTA groups and their instance lists, the exchange buffers and
// the JacobiArgs.  The stream is idle.
int layout_solve(cupic_batch *b, const Knobs &kn) {
  const int n = (int)b->members.size();
  int dev_max = 0;
  CU(cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device));
  std::vector<SimArgs> inst(n);
  std::vector<Plan> plan(n);
  std::vector<double> work(n);
  std::vector<long long> fit(n);
  size_t smem = 0;
  for (int i = 0; i < n; ++i) {
    const cupic_ctx *c = b->members[i];
    inst[i] = c->a;
    const long long P = (c->a.nnx + 3) / 4 * 4;
    const long long rows_fit = (long long)((dev_max - 1024) / (3 * sizeof(float) * P));
    fit[i] = rows_fit;
    if (!plan_instance(c->a, rows_fit, kn, &plan[i])) return CUPIC_ERR_ARG;
    smem = std::max(smem, plan[i].smem);
    work[i] = (double)c->a.nnx * c->a.nny * std::max(c->p.max_sweeps, 1);
  }
  CU(jacobi_batch_set_smem(smem));
  int per_sm = 0;
  CU(jacobi_batch_max_ctas(smem, &per_sm));
  const int T = per_sm * b->num_sms;
  // With few members the fewest CTAs that hold a mesh leave most of the GPU
  // idle: a member takes up to its share of the CTAs by work, but no more
  // than its own tuned single-context layout.  More CTAs hold fewer rows
  // each, so the shared memory per CTA does not grow.
  const double wsum = std::accumulate(work.begin(), work.end(), 0.0);
  for (int i = 0; i < n; ++i) {
    const int share = (int)(T * work[i] / wsum);
    const int want = std::min(b->members[i]->jG, share);
    Plan q;
    if (want > plan[i].G && plan_on(inst[i], want, fit[i], kn.depth, &q) && q.smem <= smem) plan[i] = q;
  }
  // buckets of equal CTA count; groups per bucket by work share
  std::vector<int> sizes;
  for (const Plan &q : plan) sizes.push_back(q.G);
  std::sort(sizes.begin(), sizes.end());
  sizes.erase(std::unique(sizes.begin(), sizes.end()), sizes.end());
  const int nb = (int)sizes.size();
  std::vector<double> bw(nb, 0.0);
  std::vector<int> bcount(nb, 0), ng(nb, 1);
  std::vector<int> bucket(n);
  for (int i = 0; i < n; ++i) {
    bucket[i] = (int)(std::lower_bound(sizes.begin(), sizes.end(), plan[i].G) - sizes.begin());
    bw[bucket[i]] += work[i];
    bcount[bucket[i]]++;
  }
  const double wtot = std::accumulate(bw.begin(), bw.end(), 0.0);
  int used = 0;
  for (int k = 0; k < nb; ++k) {
    ng[k] = std::max(1, std::min(bcount[k], (int)(T * bw[k] / wtot / sizes[k])));
    used += ng[k] * sizes[k];
  }
  while (used > T) {  // give back groups where a group carries the least work
    int kk = -1;
    for (int k = 0; k < nb; ++k)
      if (ng[k] > 1 && (kk < 0 || bw[k] / ng[k] < bw[kk] / ng[kk])) kk = k;
    if (kk < 0) return CUPIC_ERR_CAPACITY;  // one group per size does not fit the GPU
    ng[kk]--;
    used -= sizes[kk];
  }
  for (;;) {  // hand out the CTAs left where a group carries the most work
    int kk = -1;
    for (int k = 0; k < nb; ++k)
      if (ng[k] < bcount[k] && used + sizes[k] <= T && (kk < 0 || bw[k] / ng[k] > bw[kk] / ng[kk]))
        kk = k;
    if (kk < 0) break;
    ng[kk]++;
    used += sizes[kk];
  }
  // groups: consecutive CTAs; instances of a bucket go largest first to the
  // least-loaded group of the bucket
  std::vector<JGroup> groups;
  std::vector<std::vector<int>> glist;
  std::vector<double> gload;
  int first = 0;
  for (int k = 0; k < nb; ++k) {
    const int g0 = (int)groups.size();
    for (int q = 0; q < ng[k]; ++q) {
      groups.push_back({first, sizes[k], 0, 0});
      glist.emplace_back();
      gload.push_back(0.0);
      first += sizes[k];
    }
    std::vector<int> ids;
    for (int i = 0; i < n; ++i)
      if (bucket[i] == k) ids.push_back(i);
    std::sort(ids.begin(), ids.end(), [&](int x, int y) { return work[x] > work[y]; });
    for (int i : ids) {
      int best = g0;
      for (int g = g0; g < g0 + ng[k]; ++g)
        if (gload[g] < gload[best]) best = g;
      glist[best].push_back(i);
      gload[best] += work[i];
    }
  }
  std::vector<int> list;
  for (size_t g = 0; g < groups.size(); ++g) {
    groups[g].begin = (int)list.size();
    list.insert(list.end(), glist[g].begin(), glist[g].end());
    groups[g].end = (int)list.size();
  }
  b->ngroups = (int)groups.size();
  b->nctas = first;
  b->jsmem = smem;
  // exchange buffers of every instance's solve, one pool each
  size_t nflags = 0, nres = 0, nhalo = 0;
  for (int i = 0; i < n; ++i) {
    nflags += plan[i].G + 1;
    nres += 2 * plan[i].G;
    nhalo += (size_t)4 * plan[i].G * plan[i].K * plan[i].P;
  }
  int rc;
  if ((rc = grow(&b->d_flags, &b->cap_flags, nflags)) || (rc = grow(&b->d_res, &b->cap_res, nres)) ||
      (rc = grow(&b->d_halo, &b->cap_halo, nhalo)))
    return rc;
  // a region may hold another instance's words with a matching epoch
  CU(cudaMemsetAsync(b->d_halo, 0, sizeof(unsigned long long) * nhalo, b->stream));
  b->nhalo = nhalo;
  b->epoch_steps = 0;
  b->nflags = nflags;
  std::vector<JacobiArgs> jargs(n);
  size_t of = 0, orr = 0, oh = 0;
  for (int i = 0; i < n; ++i) {
    const cupic_ctx *c = b->members[i];
    const Plan &q = plan[i];
    JacobiArgs J{};
    J.tol = c->p.tol;
    J.min_sweeps = c->p.min_sweeps;
    J.max_sweeps = c->p.max_sweeps;
    J.check_every = std::max(1, c->p.check_every);
    J.G = q.G;
    J.rows_per_cta = q.B;
    J.depth = q.K;
    J.pitch = q.P;
    J.vec = ((c->a.nnx - 1) % 4 == 0) ? 1 : 0;
    J.strip = jacobi_strip_rows(c->a.nnx, q.B + 2 * (q.G > 1 ? q.K : 1) - 2);
    J.do_field = 1;
    J.write_stats = 1;
    J.zero_next = 1;  // the solve clears the accumulator the push deposits into
    J.flags = b->d_flags + of;
    J.bar = J.flags + q.G;
    J.res_cta = b->d_res + orr;
    J.halo = b->d_halo + oh;
    of += q.G + 1;
    orr += 2 * q.G;
    oh += (size_t)4 * q.G * q.K * q.P;
    jargs[i] = J;
  }
  if ((rc = grow(&b->d_groups, &b->cap_groups, groups.size()))) return rc;
  // d_jargs and d_list hold one entry per member
  cudaFree(b->d_jargs);
  cudaFree(b->d_list);
  b->d_jargs = nullptr;
  b->d_list = nullptr;
  CU(cudaMalloc(&b->d_jargs, n * sizeof(JacobiArgs)));
  CU(cudaMalloc(&b->d_list, n * sizeof(int)));
  CU(cudaMemcpy(b->d_jargs, jargs.data(), n * sizeof(JacobiArgs), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(b->d_groups, groups.data(), groups.size() * sizeof(JGroup), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(b->d_list, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice));
  b->knob_depth = kn.depth;
  b->knob_mult = kn.mult;
  return CUPIC_OK;
}

// device ms of one batched solve with the current layout: the best of two
// launches after a warm-up one
int time_solve(cupic_batch *b, float *ms) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  float best = 1e30f;
  cudaError_t e = cudaSuccess;
  for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
    e = cudaMemsetAsync(b->d_flags, 0, b->nflags * sizeof(unsigned), b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
    if (e == cudaSuccess)
      e = launch_jacobi_batch(b->d_inst, b->d_jargs, b->d_groups, b->ngroups, b->d_list, b->nctas,
                              b->jsmem, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float t = 0.0f;
    if (e == cudaSuccess && rep > 0 && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess)
      best = std::min(best, t);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *ms = 1e30f;
    return CUPIC_OK;  // the layout is left out
  }
  *ms = best;
  return CUPIC_OK;
}

// The batched-solve autotuner: times every candidate layout (halo depth cap
// x CTA multiple, kCandidates) with the members' own meshes and sweep
// counts, and keeps the fastest.  The trial solves overwrite the members'
// potential and field and their solver status words; those are saved
// before and put back after, so the members' results do not depend on the
// tuning.  The epoch base of the halo words keeps advancing, as the
// exchange protocol needs.  Picks are cached per process by the members'
// multiset of (mesh shape, sweeps), and batches of fewer than kTuneMembers
// members take the default knobs.  A batch whose members change (a server
// admitting and retiring requests) keeps its tuned knobs until its member
// count doubles or halves, so that membership changes do not tune again.
// CUPIC_BATCH_TUNE=0 turns tuning off.
struct MixKey {
  std::vector<std::tuple<int, int, int, int>> shapes;
  bool operator<(const MixKey &o) const { return shapes < o.shapes; }
};
std::mutex g_mix_mu;
std::map<std::pair<int, MixKey>, Knobs> g_mix_tuned;

int tune_solve(cupic_batch *b) {
  const int n = (int)b->members.size();
  const char *env = getenv("CUPIC_BATCH_TUNE");
  if (n < kTuneMembers || (env && atoi(env) == 0)) return layout_solve(b, kDefaultKnobs);
  if (b->tuned_n && n < 2 * b->tuned_n && 2 * n > b->tuned_n &&
      layout_solve(b, Knobs{b->knob_depth, b->knob_mult}) == CUPIC_OK)
    return CUPIC_OK;
  b->tuned_n = n;
  MixKey key;
  for (const cupic_ctx *c : b->members)
    key.shapes.emplace_back(c->a.nnx, c->a.nny, c->p.max_sweeps, c->p.check_every);
  std::sort(key.shapes.begin(), key.shapes.end());
  {
    std::lock_guard<std::mutex> lk(g_mix_mu);
    auto it = g_mix_tuned.find({b->device, key});
    if (it != g_mix_tuned.end()) return layout_solve(b, it->second);
  }
  // save what the trials overwrite
  size_t nodes = 0;
  for (const cupic_ctx *c : b->members) nodes += (size_t)c->a.nnx * c->a.nny;
  constexpr size_t kStat = offsetof(Ctl, residual) + sizeof(float) - offsetof(Ctl, step_flags);
  unsigned char *save = nullptr;
  const size_t bytes = nodes * (sizeof(float) + sizeof(float2)) + (size_t)n * (kStat + sizeof(int32_t));
  CU(cudaMalloc(&save, bytes));
  auto copy_all = [&](bool back) -> cudaError_t {
    unsigned char *q = save;
    cudaError_t e = cudaSuccess;
    for (const cupic_ctx *c : b->members) {
      const size_t nn = (size_t)c->a.nnx * c->a.nny;
      unsigned char *ctlb = reinterpret_cast<unsigned char *>(c->ctl);
      struct { void *dev; size_t len; } part[] = {
          {c->a.phi, nn * sizeof(float)}, {c->a.E, nn * sizeof(float2)},
          {ctlb + offsetof(Ctl, step_flags), kStat}, {ctlb + offsetof(Ctl, abort), sizeof(int32_t)}};
      for (auto &pt : part) {
        if (e == cudaSuccess)
          e = back ? cudaMemcpyAsync(pt.dev, q, pt.len, cudaMemcpyDeviceToDevice, b->stream)
                   : cudaMemcpyAsync(q, pt.dev, pt.len, cudaMemcpyDeviceToDevice, b->stream);
        q += pt.len;
      }
    }
    return e;
  };
  cudaError_t e = copy_all(false);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  Knobs pick = kDefaultKnobs;
  float best = 1e30f;
  int rc = e == cudaSuccess ? CUPIC_OK : CUPIC_ERR_CUDA;
  for (const Knobs &k : kCandidates) {
    if (rc) break;
    if (layout_solve(b, k) != CUPIC_OK) continue;  // this layout does not fit
    float ms = 1e30f;
    rc = time_solve(b, &ms);
    if (!rc && ms < best) {
      best = ms;
      pick = k;
    }
  }
  e = copy_all(true);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  cudaFree(save);
  if (rc) return rc;
  if (e != cudaSuccess) return CUPIC_ERR_CUDA;
  {
    std::lock_guard<std::mutex> lk(g_mix_mu);
    g_mix_tuned[{b->device, key}] = pick;
  }
  return layout_solve(b, pick);
}

int build(cupic_batch *b) {
  drop_graph(b);
  const int n = (int)b->members.size();
  b->epochs.clear();
  for (const cupic_ctx *c : b->members) b->epochs.push_back(c->layout_epoch);
  if (n == 0) return CUPIC_OK;
  std::vector<SimArgs> inst(n);
  b->max_nnx = b->max_ncy = b->max_inj = 0;
  for (int i = 0; i < n; ++i) {
    const cupic_ctx *c = b->members[i];
    inst[i] = c->a;
    b->max_nnx = std::max(b->max_nnx, c->a.nnx);
    b->max_ncy = std::max(b->max_ncy, c->a.ncy);
    b->max_inj = std::max({b->max_inj, c->a.sp[0].inj_cap, c->a.sp[1].inj_cap});
  }
  int rc;
  // work lists
  std::vector<int2> rows;
  b->max_nnx_short = b->max_nnx_mid = 0;
  b->big.clear();
  auto cls = [&](int i) { return inst[i].ncy >= kBigRows ? 2 : inst[i].ncx <= kShortRow ? 0 : 1; };
  for (int pass = 0; pass < 3; ++pass)
    for (int i = 0; i < n; ++i) {
      if (cls(i) != pass) continue;
      for (int s = 0; s < inst[i].ncy; ++s) rows.push_back(make_int2(i, s));
      if (pass == 0) b->max_nnx_short = std::max(b->max_nnx_short, inst[i].nnx);
      if (pass == 1) b->max_nnx_mid = std::max(b->max_nnx_mid, inst[i].nnx);
      if (pass == 2) b->big.push_back(i);
    }
  b->nrows_short = b->nrows_mid = 0;
  for (const int2 &r : rows) {
    if (cls(r.x) == 0) ++b->nrows_short;
    if (cls(r.x) == 1) ++b->nrows_mid;
  }
  b->nrows = (int)rows.size();
  if ((rc = grow(&b->d_inst, &b->cap_inst, (size_t)n)) || (rc = grow(&b->d_rows, &b->cap_rows, rows.size())))
    return rc;
  CU(cudaMemcpy(b->d_inst, inst.data(), n * sizeof(SimArgs), cudaMemcpyHostToDevice));
  CU(cudaMemcpy(b->d_rows, rows.data(), rows.size() * sizeof(int2), cudaMemcpyHostToDevice));
  return tune_solve(b);
}

int enqueue(cupic_batch *b) {
  const int n = (int)b->members.size();
  cudaStream_t st = b->stream;
  CU(cudaMemsetAsync(b->d_flags, 0, b->nflags * sizeof(unsigned), st));
  CU(launch_jacobi_batch(b->d_inst, b->d_jargs, b->d_groups, b->ngroups, b->d_list, b->nctas,
                         b->jsmem, st));
  CU(cudaEventRecord(b->ev_fork, st));
  CU(cudaStreamWaitEvent(b->side, b->ev_fork, 0));
  CU(launch_inject_draw_batch(b->d_inst, n, b->max_inj, b->side));
  CU(cudaEventRecord(b->ev_join, b->side));
  // big instances: the single-context push, one launch each, on parallel
  // branches beside the work-list pushes of the others
  const int nbr = b->big.empty() ? 0 : std::min(kPushBranches, (int)b->big.size());
  if (nbr) {
    CU(cudaEventRecord(b->ev_push_fork, st));
    for (int k = 0; k < nbr; ++k) CU(cudaStreamWaitEvent(b->push_st[k], b->ev_push_fork, 0));
    for (size_t q = 0; q < b->big.size(); ++q)
      CU(launch_push_deposit(b->members[b->big[q]]->a, b->push_st[q % nbr]));
    for (int k = 0; k < nbr; ++k) CU(cudaEventRecord(b->ev_push_join[k], b->push_st[k]));
  }
  CU(launch_push_deposit_batch(b->d_inst, b->d_rows, b->nrows_short, b->max_nnx_short, 128, st));
  CU(launch_push_deposit_batch(b->d_inst, b->d_rows + b->nrows_short, b->nrows_mid, b->max_nnx_mid,
                               512, st));
  for (int k = 0; k < nbr; ++k) CU(cudaStreamWaitEvent(st, b->ev_push_join[k], 0));
  CU(cudaStreamWaitEvent(st, b->ev_join, 0));
  CU(launch_room_batch(b->d_inst, n, b->max_ncy, st));
  CU(launch_arrive_batch(b->d_inst, b->d_rows, b->nrows, st));
  CU(launch_inject_append_batch(b->d_inst, n, b->max_ncy, st));
  CU(launch_finalize_batch(b->d_inst, n, st));
  return CUPIC_OK;
}

int capture(cupic_batch *b) {
  drop_graph(b);
  cudaGraph_t g = nullptr;
  CU(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const int rc = enqueue(b);
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (rc || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return CUPIC_OK;  // direct launches instead
  }
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();
    b->graph = nullptr;
    return CUPIC_OK;
  }
  b->graph_ok = true;
  return CUPIC_OK;
}

}  // namespace

extern "C" {

int cupic_batch_create(int device, cupic_batch **out) {
  if (!out) return CUPIC_ERR_ARG;
  *out = nullptr;
  cupic_batch *b = new (std::nothrow) cupic_batch();
  if (!b) return CUPIC_ERR_NOMEM;
  b->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_push_fork, cudaEventDisableTiming) != cudaSuccess) {
    cupic_batch_destroy(b);
    return CUPIC_ERR_CUDA;
  }
  for (int k = 0; k < kPushBranches; ++k)
    if (cudaStreamCreateWithFlags(&b->push_st[k], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_push_join[k], cudaEventDisableTiming) != cudaSuccess) {
      cupic_batch_destroy(b);
      return CUPIC_ERR_CUDA;
    }
  *out = b;
  return CUPIC_OK;
}

int cupic_batch_set(cupic_batch *b, cupic_ctx *const *members, int32_t n) {
  if (!b || n < 0 || (n > 0 && !members)) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(b->device));
  CU(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < n; ++i) {
    const cupic_ctx *c = members[i];
    if (!c || c->device != b->device) return CUPIC_ERR_ARG;
    if (!c->initialized || !c->rho_valid) return CUPIC_ERR_STATE;
    if (c->p.refine_every > 0) return CUPIC_ERR_ARG;  // the precision form steps alone
    for (int k = 0; k < i; ++k)
      if (members[k] == c) return CUPIC_ERR_ARG;
  }
  for (int i = 0; i < n; ++i) CU(cudaStreamSynchronize(members[i]->stream));
  b->members.assign(members, members + n);
  return build(b);
}

int cupic_batch_step(cupic_batch *b, int32_t nsteps) {
  if (!b || nsteps < 0) return CUPIC_ERR_ARG;
  if (b->members.empty() || nsteps == 0) return CUPIC_OK;
  CU(cudaSetDevice(b->device));
  // a member whose rows grew (its run halted and was completed alone) or
  // whose particles were reloaded has new buffers; a reloaded one also needs
  // the charge of its new particles
  bool rebuild = false;
  for (size_t i = 0; i < b->members.size(); ++i) {
    cupic_ctx *c = b->members[i];
    if (!c->rho_valid) {
      const int rc = cupic_charge_deposition(c);
      if (rc) return rc;
    }
    if (c->layout_epoch != b->epochs[i]) rebuild = true;
  }
  if (rebuild) {
    CU(cudaStreamSynchronize(b->stream));
    const int rc = build(b);
    if (rc) return rc;
  }
  if (!b->graph_ok) {
    int rc = capture(b);
    if (rc) return rc;
  }
  for (int s = 0; s < nsteps; ++s) {
    if (++b->epoch_steps > 65000) {  // before the members' solve counts can wrap
      CU(cudaMemsetAsync(b->d_halo, 0, sizeof(unsigned long long) * b->nhalo, b->stream));
      b->epoch_steps = 1;
    }
    if (b->graph_ok) {
      CU(cudaGraphLaunch(b->graph, b->stream));
    } else {
      int rc = enqueue(b);
      if (rc) return rc;
    }
  }
  for (cupic_ctx *c : b->members) c->host_cur ^= (nsteps & 1);
  return CUPIC_OK;
}

int cupic_batch_plan(cupic_batch *b, int32_t *depth_cap, int32_t *cta_mult, int32_t *ctas) {
  if (!b || !depth_cap || !cta_mult || !ctas) return CUPIC_ERR_ARG;
  *depth_cap = b->knob_depth;
  *cta_mult = b->knob_mult;
  *ctas = b->nctas;
  return CUPIC_OK;
}

int cupic_batch_sync(cupic_batch *b) {
  if (!b) return CUPIC_ERR_ARG;
  CU(cudaSetDevice(b->device));
  CU(cudaStreamSynchronize(b->stream));
  int first = CUPIC_OK;
  for (cupic_ctx *c : b->members) {
    const int rc = cupic_ctx_finish(c);
    if (rc && !first) first = rc;
  }
  return first;
}

int cupic_batch_destroy(cupic_batch *b) {
  if (!b) return CUPIC_ERR_ARG;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  cudaFree(b->d_inst);
  cudaFree(b->d_jargs);
  cudaFree(b->d_groups);
  cudaFree(b->d_list);
  cudaFree(b->d_rows);
  cudaFree(b->d_flags);
  cudaFree(b->d_res);
  cudaFree(b->d_halo);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->ev_push_fork) cudaEventDestroy(b->ev_push_fork);
  for (int k = 0; k < kPushBranches; ++k) {
    if (b->ev_push_join[k]) cudaEventDestroy(b->ev_push_join[k]);
    if (b->push_st[k]) {
      cudaStreamSynchronize(b->push_st[k]);
      cudaStreamDestroy(b->push_st[k]);
    }
  }
  if (b->ev_join) cudaEventDestroy(b->ev_join);
  if (b->side) {
    cudaStreamSynchronize(b->side);
    cudaStreamDestroy(b->side);
  }
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return CUPIC_OK;
}

}  // extern "C"
