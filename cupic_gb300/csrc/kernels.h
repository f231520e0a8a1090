// kernels.h -- host-side launchers of the device kernels.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "cupic_internal.cuh"

namespace cupic {

cudaError_t launch_init_particles(const SimArgs &a, cudaStream_t st);
cudaError_t launch_deposit(const SimArgs &a, cudaStream_t st);
cudaError_t launch_zero_next_rho(const SimArgs &a, cudaStream_t st);
cudaError_t launch_leapfrog_start(const SimArgs &a, cudaStream_t st);
cudaError_t launch_push_deposit(const SimArgs &a, cudaStream_t st);
cudaError_t launch_arrive(const SimArgs &a, cudaStream_t st);
cudaError_t launch_inject(const SimArgs &a, cudaStream_t st);
cudaError_t launch_finalize(const SimArgs &a, cudaStream_t st);
size_t push_smem_bytes(int nnx);
cudaError_t push_set_smem(size_t bytes);

size_t jacobi_smem_bytes(int rows_per_cta, int pitch);
int jacobi_block();
cudaError_t jacobi_set_smem(size_t bytes);
cudaError_t jacobi_max_ctas(size_t smem, int *per_sm);
cudaError_t launch_jacobi(const SimArgs &a, const JacobiArgs &J, cudaStream_t st);

}  // namespace cupic
