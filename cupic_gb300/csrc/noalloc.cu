// noalloc.cu -- the Poisson solve on caller-owned device buffers, without
// allocating any memory.
//
// Some callers cannot call cudaMalloc at the point where they need a solve:
// - a real-time loop that forbids allocation after start-up, because an
//   allocation can block for an unbounded time;
// - a host application whose device memory is all handed out by its own
//   pool, so a cudaMalloc outside that pool would fail or fragment it.
// They own the charge, potential and field buffers and just need the solve.
// The call waits for its own work (it reads the sweep count and residual
// back before returning).
//
// Such a call still needs scratch memory for the solver CTAs: per-CTA sweep
// counters, residual slots, the halo rows they trade, and a small status
// block. Here that scratch is a file-scope static device array of a fixed
// 8 MiB. Every GPU that loads this library holds it until the process
// exits. The entry point rejects meshes whose scratch would not fit.
#include <mutex>
#include <stdlib.h>
#include <string.h>

#include <algorithm>

#include "cupic_internal.cuh"
#include "kernels.h"

namespace cupic {
namespace {

constexpr size_t kStaticScratchBytes = size_t(8) << 20;
constexpr size_t kCtlHeadBytes = 256;  // the part of Ctl the solver touches
static_assert(offsetof(Ctl, ring) <= kCtlHeadBytes, "solver status block");

static __device__ __align__(256) unsigned char g_solver_scratch[kStaticScratchBytes];

// device address of g_solver_scratch for each device, looked up once
std::mutex g_mu;
constexpr int kMaxDevices = 64;
void *g_scratch_addr[kMaxDevices] = {};
// calls since the array's halo words were last zeroed, per device: a halo
// word's epoch holds the solve count in 16 bits, so the words are zeroed
// before the count can wrap (epoch 0 never matches)
long long g_calls[kMaxDevices] = {};

// the array's device address on the current device; *clear: the call must
// zero the halo words first
int scratch_for_current_device(unsigned char **out, bool *clear) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return CUPIC_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_solver_scratch) != cudaSuccess || !ptr) {
      cudaGetLastError();
      return CUPIC_ERR_CUDA;
    }
    g_scratch_addr[dev] = ptr;
  }
  *clear = ++g_calls[dev] > 65000;
  if (*clear) g_calls[dev] = 1;
  *out = static_cast<unsigned char *>(g_scratch_addr[dev]);
  return CUPIC_OK;
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace
}  // namespace cupic

using namespace cupic;

extern "C" int cupic_poisson_solver_static(const cupic_params *p, const int64_t *rho_dev,
                                           float *phi_dev, float *e_dev, double max_error,
                                           int32_t min_sweeps, int32_t max_sweeps,
                                           int32_t check_every, void *stream, int32_t *sweeps_out,
                                           float *residual_out) {
  if (!p || !rho_dev || !phi_dev || max_sweeps < 0) return CUPIC_ERR_ARG;
  if (p->ncx < 2 || p->ncy < 2 || p->ncx > 4096 || !(p->ds > 0) || !(p->eps0 > 0))
    return CUPIC_ERR_ARG;
  unsigned char *scratch = nullptr;
  bool clear_halo = false;
  int rc = scratch_for_current_device(&scratch, &clear_halo);
  if (rc) return rc;
  int dev = 0, num_sms = 0, dev_max = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return CUPIC_ERR_CUDA;

  SimArgs a{};
  a.ncx = p->ncx;
  a.ncy = p->ncy;
  a.nnx = p->ncx + 1;
  a.nny = p->ncy + 1;
  a.ds = (float)p->ds;
  a.two_ds = (float)(2.0 * p->ds);
  a.cb = ldexp(1.0, -32) / (p->ds * p->eps0);
  const int M = a.nny - 2, nnx = a.nnx;
  const int P = (nnx + 3) / 4 * 4;
  const long long rows_fit = (long long)(((size_t)dev_max - 1024) / (3 * sizeof(float) * (size_t)P));
  auto need = [&](int g, int k) {
    return kCtlHeadBytes + align256(sizeof(unsigned) * (size_t)(g + 1)) +
           align256(sizeof(float) * 2 * (size_t)g) + sizeof(unsigned long long) * (size_t)2 * g * 2 * k * P;
  };
  // one CTA when the whole mesh fits; otherwise the most CTAs (up to one per
  // SM) for which some halo depth K >= 1 fits both the CTA's shared memory
  // and the static scratch, with the deepest such K (at most 16).  The
  // library-wide tuning variable CUPIC_JACOBI_CTAS, when set, caps the CTA
  // count here as it does for a context's solve.
  const char *env = getenv("CUPIC_JACOBI_CTAS");
  const int forced = env ? atoi(env) : 0;
  int G = 0, B = 0, K = 0;
  if (forced <= 0 && M + 2 <= rows_fit && (long long)M * nnx <= 65536) {
    G = 1;
    B = M;
    K = 1;
  } else {
    const int gmax = std::max(1, std::min(forced > 0 ? forced : num_sms, M));
    for (int g = gmax; g >= 1 && K < 1; --g) {
      const int b = (M + g - 1) / g;
      int k = g > 1 ? (int)std::min<long long>({16LL, (long long)(M / g), (rows_fit - b) / 2}) : 1;
      while (k >= 1 && (need(g, k) > kStaticScratchBytes || b + 2 * k > rows_fit)) --k;
      if (k >= 1) {
        G = g;
        B = b;
        K = k;
      }
    }
    if (K < 1) return CUPIC_ERR_CAPACITY;
  }
  const size_t sm = jacobi_smem_bytes(B, K, P);
  if (jacobi_set_smem(sm) != cudaSuccess) return CUPIC_ERR_CUDA;
  int per_sm = 0;
  if (jacobi_max_ctas(sm, &per_sm) != cudaSuccess) return CUPIC_ERR_CUDA;
  if (per_sm < 1 || G > per_sm * num_sms) return CUPIC_ERR_ARG;

  // scratch layout: status block | sweep counters + barrier | residual slots | halo rows
  Ctl *ctl = reinterpret_cast<Ctl *>(scratch);
  unsigned char *q = scratch + kCtlHeadBytes;
  unsigned *flags = reinterpret_cast<unsigned *>(q);
  q += align256(sizeof(unsigned) * (size_t)(G + 1));
  float *res = reinterpret_cast<float *>(q);
  q += align256(sizeof(float) * 2 * (size_t)G);
  unsigned long long *halo = reinterpret_cast<unsigned long long *>(q);

  unsigned long long *acc = reinterpret_cast<unsigned long long *>(const_cast<int64_t *>(rho_dev));
  a.rho[0] = acc;
  a.rho[1] = acc;
  a.phi = phi_dev;
  a.E = reinterpret_cast<float2 *>(e_dev);
  a.ctl = ctl;

  JacobiArgs J{};
  J.tol = max_error;
  J.min_sweeps = min_sweeps;
  J.max_sweeps = max_sweeps;
  J.check_every = check_every < 1 ? 1 : check_every;
  J.G = G;
  J.rows_per_cta = B;
  J.depth = K;
  J.pitch = P;
  J.vec = ((nnx - 1) % 4 == 0) ? 1 : 0;
  J.strip = jacobi_strip_rows(nnx, B + 2 * (G > 1 ? K : 1) - 2);
  J.do_field = e_dev ? 1 : 0;
  J.write_stats = 1;
  J.flags = flags;
  J.bar = flags + G;
  J.res_cta = res;
  J.halo = halo;

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the array keeps the previous call's contents: clear the status block
  // (charge index 0, no abort, no flags) but not the epoch base, which
  // keeps the halo words of earlier calls from matching; launch_jacobi
  // clears the counters
  if (cudaMemsetAsync(ctl, 0, offsetof(Ctl, jepoch), st) != cudaSuccess) return CUPIC_ERR_CUDA;
  if (clear_halo && cudaMemsetAsync(scratch + kCtlHeadBytes, 0, kStaticScratchBytes - kCtlHeadBytes, st) !=
                        cudaSuccess)
    return CUPIC_ERR_CUDA;
  if (launch_jacobi(a, J, st) != cudaSuccess) return CUPIC_ERR_CUDA;
  struct {
    uint32_t step_flags;
    int32_t sweeps;
    float residual;
  } out;
  static_assert(offsetof(Ctl, sweeps) == offsetof(Ctl, step_flags) + 4, "Ctl layout");
  static_assert(offsetof(Ctl, residual) == offsetof(Ctl, sweeps) + 4, "Ctl layout");
  if (cudaMemcpyAsync(&out, &ctl->step_flags, sizeof(out), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return CUPIC_ERR_CUDA;
  if (sweeps_out) *sweeps_out = out.sweeps;
  if (residual_out) *residual_out = out.residual;
  if (out.step_flags & CUPIC_FLAG_TIMEOUT) return CUPIC_ERR_TIMEOUT;
  return CUPIC_OK;
}
