// ctx.h -- the host-side state of one context (cupic_ctx), shared by the
// C-ABI (capi.cu) and the batched form (batch.cu).
#pragma once

#include <stdint.h>

#include <vector>

#include "cupic_internal.cuh"

using cupic::Ctl;
using cupic::SimArgs;

struct cupic_ctx {
  cupic_params p;
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  // side branch of a step: the injection draws run beside the push
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  SimArgs a{};
  Ctl *ctl = nullptr;
  std::vector<int64_t> seg[2];
  std::vector<int32_t> cap[2];
  int64_t total_cap[2] = {0, 0};
  // Jacobi geometry and exchange buffers
  int jG = 1, jB = 1, jK = 1, jP = 0;
  bool jNoStrip = false;  // the tuner found the shared-memory sweep faster than register strips
  unsigned *jflags = nullptr;  // [G+1]: per-CTA sweep counters, then the barrier
  float *jres = nullptr;
  unsigned long long *jhalo = nullptr;  // halo words, zeroed at allocation
  size_t jhalo_words = 0;
  // solves enqueued since the halo words were last zeroed (see epoch_guard)
  int64_t epoch_solves = 0;
  // precision form of the solve (refine_every > 0): FP64 potential, FP32
  // residual source and correction, the residual's max norm
  double *phi64 = nullptr;
  double *b64 = nullptr;  // the FP64 source of the running solve
  float *rr = nullptr, *dl = nullptr;
  unsigned long long *maxr = nullptr;
  void *h_pin = nullptr;  // pinned: [0] max-norm bits, [1] {sweeps, residual}
  // scratch of the host-format particle transfers, grown on demand and kept
  void *io_buf = nullptr;
  size_t io_cap = 0;
  // graph of one step
  cudaGraphExec_t graph = nullptr;
  bool graph_ok = false;
  bool initialized = false;
  bool rho_valid = false;
  int host_cur = 0;
  // advanced whenever rows or staging rows move to new buffers (a batch
  // holding this context's SimArgs rebuilds)
  int layout_epoch = 0;
  // CUPIC_FLAG_* raised on the host: a halted run whose rows could not grow
  // (no memory, or a row past 2^31 places) stays halted and reports
  // CUPIC_FLAG_CAPACITY with the device's flags until the flags are cleared
  uint32_t host_flags = 0;
  int grow_status = 0;  // the status that growth failed with
};

// status helpers of capi.cu used by batch.cu
int cupic_ctx_finish(cupic_ctx *c);
