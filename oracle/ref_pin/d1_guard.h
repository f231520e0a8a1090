/* Forced include for the reference's src/mesh.cu only.  mesh.cu:480-494
 * defines atomicAdd(double*, double), which sm_60+ already provides (defect
 * D1), so its own copy is renamed after the CUDA headers are in.  TEST
 * INFRASTRUCTURE ONLY. */
#include <cuda_runtime.h>
#define atomicAdd cupic_ref_dp_atomicAdd
