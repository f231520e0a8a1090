// refine.cu -- the precision form of the Poisson solve: FP32 Jacobi sweeps
// on a correction, with the residual, the update and the field in FP64.
//
// The 5-point Jacobi iteration is linear, so m sweeps from phi equal phi
// plus m sweeps from 0 on A d = r, r = b - A phi.  The potential is held in
// FP64; every m sweeps the residual of the FP64 potential is formed in FP64
// (the true residual of the 5-point operator, max norm reported), the
// FP32 Jacobi kernel runs m sweeps on the correction with r as its source,
// and the correction is added in FP64.  The FP32 rounding then only touches
// the correction, which shrinks with the residual, so the potential reaches
// FP64 accuracy.  Operator, seam and boundary rows as in the Jacobi kernel
// (mesh.cu:327-350): columns 0 .. nnx-2 are unknowns, column nnx-1 mirrors
// column 0, the west neighbour of column 0 is column nnx-2, rows 0 and
// nny-1 are Dirichlet.
#include "cupic_internal.cuh"
#include "kernels.h"

namespace cupic {

namespace {

constexpr int kRBlock = 256;

// source b of node (i, j) in FP64 from the raw charge accumulator
__device__ __forceinline__ double source64(const SimArgs &a, const long long *acc, size_t rb, int i) {
  const int nnx = a.nnx;
  const long long f = (i == 0 || i == nnx - 1) ? acc[rb] + acc[rb + nnx - 1] : acc[rb + i];
  return (double)f * a.cb;
}

// the FP64 source of every node, once per solve (0 on the Dirichlet rows)
__global__ void __launch_bounds__(kRBlock) k_r64_source(SimArgs a, double *b64) {
  if (halted(a.ctl)) return;
  const int j = blockIdx.y, nnx = a.nnx, nny = a.nny;
  const size_t rb = (size_t)j * nnx;
  const long long *acc = reinterpret_cast<const long long *>(a.rho[a.ctl->cur]);
  for (int i = blockIdx.x * kRBlock + threadIdx.x; i < nnx; i += gridDim.x * kRBlock)
    b64[rb + i] = (j == 0 || j == nny - 1) ? 0.0 : source64(a, acc, rb, i == nnx - 1 ? 0 : i);
}

// r = b - A phi64 on interior rows (FP32 copy in rr, max |r| into *maxr as
// the bits of a non-negative double)
__global__ void __launch_bounds__(kRBlock) k_r64_residual(SimArgs a, const double *phi64, const double *b64,
                                                         float *rr, unsigned long long *maxr, int gated) {
  if (halted(a.ctl) || (gated && *reinterpret_cast<volatile int *>(&a.ctl->refine_done))) return;
  const int j = blockIdx.y, nnx = a.nnx, nny = a.nny;
  const size_t rb = (size_t)j * nnx;
  double m = 0.0;
  for (int i = blockIdx.x * kRBlock + threadIdx.x; i < nnx; i += gridDim.x * kRBlock) {
    if (j == 0 || j == nny - 1) {
      rr[rb + i] = 0.0f;
      continue;
    }
    const int ii = i == nnx - 1 ? 0 : i;  // the mirror column carries column 0's residual
    const double c = phi64[rb + ii];
    const double w = phi64[rb + (ii == 0 ? nnx - 2 : ii - 1)];
    const double e = phi64[rb + ii + 1];
    const double n = phi64[rb + nnx + ii], s = phi64[rb - nnx + ii];
    const double r = b64[rb + ii] - (4.0 * c - (((w + e) + n) + s));
    rr[rb + i] = __double2float_rn(r);
    m = fmax(m, fabs(r));
  }
  // max over the block, then one atomic per block (order independent)
  __shared__ double red[kRBlock / 32];
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kRBlock / 32; ++w) m = fmax(m, red[w]);
    atomicMax(maxr, (unsigned long long)__double_as_longlong(m));
  }
}

// phi64 += dl on interior rows (the FP32 potential follows once, at the end
// of the solve)
__global__ void __launch_bounds__(kRBlock) k_r64_update(SimArgs a, double *phi64, const float *dl, int gated) {
  if (halted(a.ctl) || (gated && *reinterpret_cast<volatile int *>(&a.ctl->refine_done))) return;
  const int j = blockIdx.y, nnx = a.nnx;
  if (j < 1 || j > a.nny - 2) return;
  const size_t rb = (size_t)j * nnx;
  for (int i = blockIdx.x * kRBlock + threadIdx.x; i < nnx; i += gridDim.x * kRBlock)
    phi64[rb + i] += (double)dl[rb + i];
}

// the FP32 potential from phi64, at the end of a solve
__global__ void __launch_bounds__(kRBlock) k_r64_phi32(SimArgs a, const double *phi64) {
  if (halted(a.ctl)) return;
  const size_t rb = (size_t)blockIdx.y * a.nnx;
  for (int i = blockIdx.x * kRBlock + threadIdx.x; i < a.nnx; i += gridDim.x * kRBlock)
    a.phi[rb + i] = __double2float_rn(phi64[rb + i]);
}

// the stop test of the precision form after `sweeps` correction sweeps, on
// the device: stop when the FP64 residual's max norm is below tol after at
// least mn sweeps, or at mx sweeps; the first test that stops sets
// refine_done (the later corrections then return at once) and records the
// solve's sweeps and residual
__global__ void k_r64_decide(Ctl *ctl, const unsigned long long *maxr, int sweeps, int mn, int mx,
                             double tol, int write_stats) {
  if (ctl->refine_done || halted(ctl)) return;
  const double res = __longlong_as_double((long long)*maxr);
  if ((sweeps >= mn && res < tol) || sweeps >= mx) {
    ctl->refine_done = 1;
    if (write_stats) {
      ctl->sweeps = sweeps;
      ctl->residual = (float)res;
    }
  }
}

// E = -grad phi from phi64 (mesh.cu:413-468), rounded once to FP32
__global__ void __launch_bounds__(kRBlock) k_r64_field(SimArgs a, const double *phi64) {
  if (halted(a.ctl)) return;
  const int j = blockIdx.y, nnx = a.nnx, nny = a.nny;
  const size_t rb = (size_t)j * nnx;
  for (int i = blockIdx.x * kRBlock + threadIdx.x; i < nnx; i += gridDim.x * kRBlock) {
    const size_t k = rb + i;
    double ex = 0.0, ey;
    if (j == 0) {
      ey = (phi64[k] - phi64[k + nnx]) / a.ds_d;
    } else if (j == nny - 1) {
      ey = (phi64[k - nnx] - phi64[k]) / a.ds_d;
    } else {
      const bool seam = i == 0 || i == nnx - 1;
      const double w = seam ? phi64[rb + nnx - 2] : phi64[k - 1];
      const double e = seam ? phi64[rb + 1] : phi64[k + 1];
      ex = (w - e) / (2.0 * a.ds_d);
      ey = (phi64[k - nnx] - phi64[k + nnx]) / (2.0 * a.ds_d);
    }
    a.E[k] = make_float2(__double2float_rn(ex), __double2float_rn(ey));
    a.phi[k] = __double2float_rn(phi64[k]);
  }
}

dim3 row_grid(const SimArgs &a) { return dim3((a.nnx + kRBlock - 1) / kRBlock, a.nny); }

}  // namespace

cudaError_t launch_r64_source(const SimArgs &a, double *b64, cudaStream_t st) {
  k_r64_source<<<row_grid(a), kRBlock, 0, st>>>(a, b64);
  return cudaGetLastError();
}

cudaError_t launch_r64_residual(const SimArgs &a, const double *phi64, const double *b64, float *rr,
                                unsigned long long *maxr, cudaStream_t st, int gated) {
  cudaError_t e = cudaMemsetAsync(maxr, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  k_r64_residual<<<row_grid(a), kRBlock, 0, st>>>(a, phi64, b64, rr, maxr, gated);
  return cudaGetLastError();
}

cudaError_t launch_r64_phi32(const SimArgs &a, const double *phi64, cudaStream_t st) {
  k_r64_phi32<<<row_grid(a), kRBlock, 0, st>>>(a, phi64);
  return cudaGetLastError();
}

cudaError_t launch_r64_update(const SimArgs &a, double *phi64, const float *dl, cudaStream_t st,
                              int gated) {
  k_r64_update<<<row_grid(a), kRBlock, 0, st>>>(a, phi64, dl, gated);
  return cudaGetLastError();
}

cudaError_t launch_r64_decide(const SimArgs &a, const unsigned long long *maxr, int sweeps, int mn,
                              int mx, double tol, int write_stats, cudaStream_t st) {
  k_r64_decide<<<1, 1, 0, st>>>(a.ctl, maxr, sweeps, mn, mx, tol, write_stats);
  return cudaGetLastError();
}

cudaError_t launch_r64_field(const SimArgs &a, const double *phi64, cudaStream_t st) {
  k_r64_field<<<row_grid(a), kRBlock, 0, st>>>(a, phi64);
  return cudaGetLastError();
}

}  // namespace cupic
