/* Forced include for the reference's src/init.cu and src/diagnostic.cu in
 * the file pin (ref_pin.build_files): their cudaMalloc and cudaMemcpy calls
 * act on host memory, so the reference's particle-file reader and its
 * snapshot writers run on the CPU without a GPU.  TEST INFRASTRUCTURE ONLY. */
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>
static inline cudaError_t cupic_ref_host_malloc(void **p, size_t n) {
  *p = calloc(1, n + 256);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
static inline cudaError_t cupic_ref_host_memcpy(void *d, const void *s, size_t n) {
  memcpy(d, s, n);
  return cudaSuccess;
}
#define cudaMalloc(p, n) cupic_ref_host_malloc((void **)(p), (n))
#define cudaMemcpy(d, s, n, k) cupic_ref_host_memcpy((d), (s), (n))
