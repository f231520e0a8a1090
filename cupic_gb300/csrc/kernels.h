// kernels.h -- host-side launchers of the device kernels.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "cupic_internal.cuh"

namespace cupic {

// Raises a kernel's dynamic shared memory limit on the current device to at
// least `bytes`.  The attribute is per device, so the largest size set so
// far is kept per (kernel, device), under a lock; it only grows, so
// contexts of different sizes coexist.
cudaError_t raise_dyn_smem(const void *kernel, size_t bytes);

cudaError_t launch_init_particles(const SimArgs &a, cudaStream_t st);
cudaError_t launch_deposit(const SimArgs &a, cudaStream_t st);
cudaError_t launch_zero_next_rho(const SimArgs &a, cudaStream_t st);
cudaError_t launch_leapfrog_start(const SimArgs &a, cudaStream_t st);
cudaError_t launch_push_deposit(const SimArgs &a, cudaStream_t st);
cudaError_t launch_arrive(const SimArgs &a, cudaStream_t st);
cudaError_t launch_inject_draw(const SimArgs &a, cudaStream_t st);
cudaError_t launch_inject_append(const SimArgs &a, cudaStream_t st);
cudaError_t launch_finalize(const SimArgs &a, cudaStream_t st);
// room check between the push and the arrivals (sets ctl->halt), and the
// move of a species' rows into a larger layout
cudaError_t launch_room(const SimArgs &a, cudaStream_t st);
cudaError_t launch_move_rows(const float4 *old, const int64_t *oseg, float4 *parts, const int64_t *nseg,
                             const int32_t *keep, int ncy, cudaStream_t st);
size_t push_smem_bytes(int nnx, int pb = 256);  // pb: threads per block (256 single context)
cudaError_t push_set_smem(size_t bytes);
// set-up on the context's stream
cudaError_t launch_uniform_layout(const SpeciesDev &S, int ncy, int capj, cudaStream_t st);
cudaError_t launch_set_time(Ctl *ctl, int64_t step, double t, double tin_e, double tin_i, cudaStream_t st);
cudaError_t launch_linear_phi(const SimArgs &a, double phi_p, double *phi64, cudaStream_t st);

int load_blocks(int64_t n, int num_sms);
cudaError_t launch_load_hist(const SimArgs &a, const double *in, int64_t n, int nb, float4 *tmp,
                             int32_t *H, unsigned *bad, cudaStream_t st);
cudaError_t launch_load_scan(int32_t *H, int nb, int ncy, int32_t *cnt, cudaStream_t st);
cudaError_t launch_load_scatter(const SimArgs &a, int sp, const float4 *tmp, int64_t n, int nb,
                                const int32_t *H, cudaStream_t st);
cudaError_t launch_pack_rows(const SimArgs &a, int sp, const int64_t *off, float4 *out32,
                             double *out64, cudaStream_t st);

size_t jacobi_smem_bytes(int rows_per_cta, int depth, int pitch);
int jacobi_strip_rows(int nnx, int urows);
cudaError_t jacobi_set_smem(size_t bytes);
cudaError_t jacobi_max_ctas(size_t smem, int *per_sm);
cudaError_t launch_jacobi(const SimArgs &a, const JacobiArgs &J, cudaStream_t st);

// many contexts in one launch (batch.cu): SimArgs / JacobiArgs arrays in
// device memory, work lists of {instance, row}
cudaError_t jacobi_batch_set_smem(size_t bytes);
cudaError_t jacobi_batch_max_ctas(size_t smem, int *per_sm);
cudaError_t launch_jacobi_batch(const SimArgs *inst, const JacobiArgs *jargs, const JGroup *groups,
                                int ngroups, const int *list, int nctas, size_t smem, cudaStream_t st);
cudaError_t launch_push_deposit_batch(const SimArgs *inst, const int2 *row_work, int n, int max_nnx,
                                      int threads, cudaStream_t st);
cudaError_t launch_arrive_batch(const SimArgs *inst, const int2 *row_work, int n, cudaStream_t st);
cudaError_t launch_inject_draw_batch(const SimArgs *inst, int n, int max_inj_cap, cudaStream_t st);
cudaError_t launch_inject_append_batch(const SimArgs *inst, int n, int max_ncy, cudaStream_t st);
cudaError_t launch_room_batch(const SimArgs *inst, int n, int max_ncy, cudaStream_t st);
cudaError_t launch_finalize_batch(const SimArgs *inst, int n, cudaStream_t st);

// fault-detection self-test (jacobi.cu)
cudaError_t launch_wait_probe(const SimArgs &a, cudaStream_t st);

// precision form of the solve (refine.cu)
// gated: the kernel returns at once when the device-side stop test has passed
cudaError_t launch_r64_source(const SimArgs &a, double *b64, cudaStream_t st);
cudaError_t launch_r64_residual(const SimArgs &a, const double *phi64, const double *b64, float *rr,
                                unsigned long long *maxr, cudaStream_t st, int gated = 0);
cudaError_t launch_r64_phi32(const SimArgs &a, const double *phi64, cudaStream_t st);
cudaError_t launch_r64_update(const SimArgs &a, double *phi64, const float *dl, cudaStream_t st,
                              int gated = 0);
cudaError_t launch_r64_decide(const SimArgs &a, const unsigned long long *maxr, int sweeps, int mn,
                              int mx, double tol, int write_stats, cudaStream_t st);
cudaError_t launch_r64_field(const SimArgs &a, const double *phi64, cudaStream_t st);

}  // namespace cupic
