// jacobi.cu -- Poisson solve (5-point Jacobi, periodic in x, Dirichlet in y)
// with the field derivation fused into the end of the last sweep
// (reference: jacobi_iteration mesh.cu:297-381, its host loop
// mesh.cu:55-120, field_derivation mesh.cu:385-472).
//
// The potential stays resident in shared memory for the whole solve: CTA c
// of a cooperative grid of G CTAs owns interior node rows [r0, r1) and keeps
// them, one halo row on each side, in two shared buffers (true Jacobi, not
// the reference's in-place update, defect D5).  After every sweep each CTA
// publishes its first and last row to an L2-resident exchange buffer and
// raises a per-CTA sweep counter; a CTA waits only for its two neighbours.
// Convergence checks use a grid barrier, and every wait is bounded: when a
// wait gives up the kernel raises CUPIC_FLAG_TIMEOUT and all CTAs return.
#include <math.h>

#include "cupic_internal.cuh"
#include "kernels.h"

namespace cupic {

namespace {

constexpr int kJBlock = 1024;
constexpr long long kSpinLimit = 1ll << 22;

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// spin until *p >= v; false if the wait gave up or another CTA aborted
__device__ bool wait_geq(const unsigned *p, unsigned v, Ctl *ctl) {
  for (long long it = 0; it < kSpinLimit; ++it) {
    if (ld_acquire(p) >= v) return true;
    if ((it & 255) == 255 && *(volatile int *)&ctl->abort) return false;
    if (it > 4096) __nanosleep(32);
  }
  atomicExch(&ctl->abort, 1);
  atomicOr(&ctl->step_flags, (uint32_t)CUPIC_FLAG_TIMEOUT);
  return false;
}

__device__ __forceinline__ float block_max(float v, float *red) {
  v = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(v)));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    float w = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0f;
    w = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(w)));
    if (lane == 0) red[32] = w;
  }
  __syncthreads();
  return red[32];
}

}  // namespace

struct SweepGeom {
  int P, W, NG, TPR, RPI, gx, gy, lane;
};

// One Jacobi sweep of local rows [u0, u1) from S into D (mesh.cu:327-350):
// v = 1/4 ((((b + west) + east) + north) + south), column nnx-1 mirroring
// column 0 and the west neighbour of column 0 being column nnx-2.  Thread
// (gx, gy) computes the 4 nodes 4gx..4gx+3 of rows u0+gy, u0+gy+RPI, ...;
// its west/east neighbours come from the adjacent lanes by shuffle, or from
// shared memory at the ends of a warp or a row.  The trip count is uniform
// across each warp (rows advance by RPI from a common base), so the
// shuffles always see all 32 lanes.  Returns the max |v - old| over owned
// rows when CHECK.
template <bool CHECK>
__device__ __forceinline__ float sweep_vec(const float *__restrict__ S, float *__restrict__ D,
                                           const float *__restrict__ bsrc, const SweepGeom &g, int u0,
                                           int u1, int o0, int o1) {
  const int P = g.P, W = g.W;
  const int col = g.gx << 2;
  const bool lfix = g.lane == 0 || g.gx == 0;
  const bool rfix = g.lane == 31 || g.gx == g.TPR - 1;
  const bool seam = g.gx == 0;
  const int lcol = seam ? W - 1 : col - 1;
  const bool active = g.gy < g.RPI;
  float md = 0.0f;
  for (int base = u0; base < u1; base += g.RPI) {
    const int lr = base + g.gy;
    const bool ok = active && lr < u1;
    const float *rowp = S + lr * P;
    float4 c4 = make_float4(0.f, 0.f, 0.f, 0.f), n4 = c4, s4 = c4, b4 = c4;
    if (ok) {
      c4 = *reinterpret_cast<const float4 *>(rowp + col);
      n4 = *reinterpret_cast<const float4 *>(rowp + P + col);
      s4 = *reinterpret_cast<const float4 *>(rowp - P + col);
      b4 = *reinterpret_cast<const float4 *>(bsrc + lr * P + col);
    }
    float lf = __shfl_up_sync(0xffffffffu, c4.w, 1);
    float rt = __shfl_down_sync(0xffffffffu, c4.x, 1);
    if (ok) {
      if (lfix) lf = rowp[lcol];
      if (rfix) rt = rowp[col + 4];  // col+4 == W is the seam copy of node 0
      float4 v;
      v.x = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(b4.x, lf), c4.y), n4.x), s4.x));
      v.y = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(b4.y, c4.x), c4.z), n4.y), s4.y));
      v.z = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(b4.z, c4.y), c4.w), n4.z), s4.z));
      v.w = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(b4.w, c4.z), rt), n4.w), s4.w));
      float *dp = D + lr * P;
      *reinterpret_cast<float4 *>(dp + col) = v;
      if (seam) dp[W] = v.x;
      if (CHECK && lr >= o0 && lr < o1) {
        md = fmaxf(md, fabsf(__fsub_rn(v.x, c4.x)));
        md = fmaxf(md, fabsf(__fsub_rn(v.y, c4.y)));
        md = fmaxf(md, fabsf(__fsub_rn(v.z, c4.z)));
        md = fmaxf(md, fabsf(__fsub_rn(v.w, c4.w)));
        if (seam) md = fmaxf(md, fabsf(__fsub_rn(v.x, rowp[W])));
      }
    }
  }
  return md;
}

// the same sweep, one node per thread (used when (nnx-1) % 4 != 0)
template <bool CHECK>
__device__ __forceinline__ float sweep_scalar(const float *__restrict__ S, float *__restrict__ D,
                                              const float *__restrict__ bsrc, const SweepGeom &g,
                                              int u0, int u1, int o0, int o1) {
  const int P = g.P, W = g.W;
  float md = 0.0f;
  if (g.gy >= g.RPI) return md;
  for (int lr = u0 + g.gy; lr < u1; lr += g.RPI) {
    const float *cr = S + lr * P;
    for (int i = g.gx; i < W; i += g.TPR) {
      const float wv = (i == 0) ? cr[W - 1] : cr[i - 1];
      const float v = __fmul_rn(
          0.25f, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(bsrc[lr * P + i], wv), cr[i + 1]), cr[P + i]),
                           cr[i - P]));
      D[lr * P + i] = v;
      const bool own = CHECK && lr >= o0 && lr < o1;
      if (own) md = fmaxf(md, fabsf(__fsub_rn(v, cr[i])));
      if (i == 0) {
        D[lr * P + W] = v;
        if (own) md = fmaxf(md, fabsf(__fsub_rn(v, cr[W])));
      }
    }
  }
  return md;
}

// Rows of CTA c: interior rows [r0, r1) with r0 = 1 + c*M/G (M = nny-2), so
// every CTA owns floor(M/G) or ceil(M/G) rows.  With temporal blocking depth
// k, a CTA also holds k halo rows on each side; sweep m (1..k) after an
// exchange updates the rows [r0-k+m, r1+k-m) -- the halo part redundantly,
// with the same operands as the neighbour, so the values are identical --
// and the neighbours trade their k boundary rows only every k sweeps.
__global__ void __launch_bounds__(kJBlock, 1) k_jacobi(SimArgs a, JacobiArgs J) {
  extern __shared__ float jsm[];
  __shared__ float red[33];
  __shared__ int bail;
  const int c = blockIdx.x, G = J.G, tid = threadIdx.x;
  const int nnx = a.nnx, nny = a.nny, P = J.pitch;
  const int M = nny - 2;
  const int K = G > 1 ? J.depth : 1;
  const int r0 = 1 + (int)(((long long)c * M) / G);
  const int r1 = 1 + (int)(((long long)(c + 1) * M) / G);
  const int lo = max(0, r0 - K);             // first buffered row
  const int hi = min(nny - 1, r1 - 1 + K);   // last buffered row
  const int nrows = hi - lo + 1;
  const int cap = J.rows_per_cta + 2 * K;    // buffer rows reserved per array
  float *const buf0 = jsm;
  float *const buf1 = jsm + (size_t)cap * P;
  float *const bsrc = jsm + (size_t)2 * cap * P;  // same row indexing as the buffers
  Ctl *ctl = a.ctl;
  if (tid == 0) bail = 0;

  const long long *acc = reinterpret_cast<const long long *>(a.rho[ctl->cur]);
  for (int lr = 0; lr < nrows; ++lr) {
    const int j = lo + lr;
    const size_t rb = (size_t)j * nnx;
    const bool interior = j >= 1 && j <= nny - 2;
    for (int i = tid; i < nnx; i += kJBlock) {
      const float v = a.phi[rb + i];
      buf0[lr * P + i] = v;
      buf1[lr * P + i] = v;
      if (interior) {
        const long long f = (i == 0 || i == nnx - 1) ? acc[rb] + acc[rb + nnx - 1] : acc[rb + i];
        bsrc[lr * P + i] = __double2float_rn((double)f * a.cb);
      }
    }
  }
  __syncthreads();

  const int W = nnx - 1;  // computed columns 0 .. nnx-2; column nnx-1 mirrors 0
  const bool vec = J.vec != 0;
  SweepGeom sg;
  sg.P = P;
  sg.W = W;
  sg.NG = vec ? (W >> 2) : W;  // column groups per row (4 nodes each on the vector path)
  sg.TPR = min(sg.NG, kJBlock);
  sg.RPI = kJBlock / sg.TPR;
  sg.gx = tid % sg.TPR;
  sg.gy = tid / sg.TPR;
  sg.lane = tid & 31;
  const int o0 = r0 - lo, o1 = r1 - lo;  // owned local rows
  auto sweep = [&](const float *S, float *D, int u0, int u1, bool check) -> float {
    if (u0 >= u1) return 0.0f;
    if (vec) return check ? sweep_vec<true>(S, D, bsrc, sg, u0, u1, o0, o1)
                          : sweep_vec<false>(S, D, bsrc, sg, u0, u1, o0, o1);
    return check ? sweep_scalar<true>(S, D, bsrc, sg, u0, u1, o0, o1)
                 : sweep_scalar<false>(S, D, bsrc, sg, u0, u1, o0, o1);
  };
  // halo exchange, split in two so the rows that need no halo can be swept
  // while the neighbours' rows are in flight
  auto publish = [&](const float *D, int e) {
    float *hp = J.halo + ((size_t)(e & 1) * G + c) * 2 * K * P;
    for (int r = 0; r < K; ++r)
      for (int i = tid; i < nnx; i += kJBlock) {
        __stcg(hp + r * P + i, D[(o0 + r) * P + i]);
        __stcg(hp + (K + r) * P + i, D[(o1 - K + r) * P + i]);
      }
    __syncthreads();
    if (tid == 0) st_release(&J.flags[c], (unsigned)e);
  };
  auto receive = [&](float *D, int e) -> bool {
    if (tid == 0) {
      bool ok = true;
      if (c > 0) ok = wait_geq(&J.flags[c - 1], (unsigned)e, ctl);
      if (ok && c < G - 1) ok = wait_geq(&J.flags[c + 1], (unsigned)e, ctl);
      if (!ok) bail = 1;
    }
    __syncthreads();
    if (bail) return false;
    if (c > 0) {  // rows [r0-K, r0) = the lower neighbour's last K rows
      const float *hn = J.halo + ((size_t)(e & 1) * G + (c - 1)) * 2 * K * P + K * P;
      for (int r = 0; r < K; ++r)
        for (int i = tid; i < nnx; i += kJBlock) D[(o0 - K + r) * P + i] = __ldcg(hn + r * P + i);
    }
    if (c < G - 1) {  // rows [r1, r1+K) = the upper neighbour's first K rows
      const float *hn = J.halo + ((size_t)(e & 1) * G + (c + 1)) * 2 * K * P;
      for (int r = 0; r < K; ++r)
        for (int i = tid; i < nnx; i += kJBlock) D[(o1 + r) * P + i] = __ldcg(hn + r * P + i);
    }
    __syncthreads();
    return true;
  };

  int src = 0, done = 0, nchk = 0, m = 0, pending = 0, to_check = J.check_every;
  float last = INFINITY;
  for (int s = 1; s <= J.max_sweeps; ++s) {
    float *S = src ? buf1 : buf0;
    float *D = src ? buf0 : buf1;
    const bool check = (--to_check == 0) || (s == J.max_sweeps);
    if (to_check == 0) to_check = J.check_every;
    m = (m >= K) ? 1 : m + 1;                        // position in the temporal block
    const int u0 = max(1, r0 - K + m) - lo;          // updated local rows [u0, u1)
    const int u1 = min(nny - 2, r1 - 1 + K - m) + 1 - lo;
    float md;
    if (pending) {
      // rows o0+1 .. o1-2 read only owned rows of S: sweep them first
      const int i0 = max(u0, o0 + 1), i1 = min(u1, o1 - 1);
      md = sweep(S, D, i0, i1, check);
      if (!receive(S, pending)) break;
      md = fmaxf(md, sweep(S, D, u0, min(i0, u1), check));
      md = fmaxf(md, sweep(S, D, max(i1, u0), u1, check));
      pending = 0;
    } else {
      md = sweep(S, D, u0, u1, check);
    }
    __syncthreads();
    if (G > 1 && m == K) {
      publish(D, s / K);
      pending = s / K;
    }
    src ^= 1;
    done = s;
    if (check) {
      float bm = block_max(md, red);
      if (G > 1) {
        if (tid == 0) {
          __stcg(&J.res_cta[(nchk & 1) * G + c], bm);
          __threadfence();
          atomicAdd(J.bar, 1u);
          if (!wait_geq(J.bar, (unsigned)(G * (nchk + 1)), ctl)) bail = 1;
        }
        __syncthreads();
        if (bail) break;
        float v = 0.0f;
        for (int k = tid; k < G; k += kJBlock) v = fmaxf(v, __ldcg(&J.res_cta[(nchk & 1) * G + k]));
        bm = block_max(v, red);
      }
      ++nchk;
      last = bm;
      if (s >= J.min_sweeps && (double)bm < J.tol) break;
    }
  }
  float *F = src ? buf1 : buf0;
  if (pending && !bail) receive(F, pending);

  // write back the owned rows; derive E = -grad phi (mesh.cu:413-468).  The
  // rows r0-1 and r1 are current: either just exchanged or updated in the
  // last sweep of an unfinished temporal block.
  for (int lr = o0; lr < o1; ++lr)
    for (int i = tid; i < nnx; i += kJBlock) a.phi[(size_t)(lo + lr) * nnx + i] = F[lr * P + i];
  if (J.do_field) {
    for (int lr = o0; lr < o1; ++lr) {
      const float *cr = F + lr * P;
      for (int i = tid; i < nnx; i += kJBlock) {
        const bool seam = (i == 0 || i == nnx - 1);
        const float wv = seam ? cr[nnx - 2] : cr[i - 1];
        const float ev = seam ? cr[1] : cr[i + 1];
        float2 e;
        e.x = __fdiv_rn(__fsub_rn(wv, ev), a.two_ds);
        e.y = __fdiv_rn(__fsub_rn(cr[i - P], cr[i + P]), a.two_ds);
        a.E[(size_t)(lo + lr) * nnx + i] = e;
      }
    }
    if (c == 0) {
      for (int i = tid; i < nnx; i += kJBlock)
        a.E[i] = make_float2(0.0f, __fdiv_rn(__fsub_rn(F[i], F[P + i]), a.ds));
    }
    if (c == G - 1) {
      const int t = (nny - 1) - lo;
      for (int i = tid; i < nnx; i += kJBlock)
        a.E[(size_t)(nny - 1) * nnx + i] =
            make_float2(0.0f, __fdiv_rn(__fsub_rn(F[(t - 1) * P + i], F[t * P + i]), a.ds));
    }
  }
  if (J.write_stats && c == 0 && tid == 0) {
    ctl->sweeps = done;
    ctl->residual = last;
  }
}

size_t jacobi_smem_bytes(int rows_per_cta, int depth, int pitch) {
  return (size_t)3 * (rows_per_cta + 2 * depth) * pitch * sizeof(float);
}

int jacobi_block() { return kJBlock; }

// the attribute only grows, so contexts of different sizes can coexist
cudaError_t jacobi_set_smem(size_t bytes) {
  static size_t cur = 0;
  if (bytes <= cur) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

cudaError_t jacobi_max_ctas(size_t smem, int *per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_jacobi, kJBlock, smem);
}

cudaError_t launch_jacobi(const SimArgs &a, const JacobiArgs &J, cudaStream_t st) {
  const size_t sm = jacobi_smem_bytes(J.rows_per_cta, J.G > 1 ? J.depth : 1, J.pitch);
  if (J.G > 1) {
    cudaError_t e = cudaMemsetAsync(J.flags, 0, sizeof(unsigned) * (J.G + 1), st);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(J.G);
  cfg.blockDim = dim3(kJBlock);
  cfg.dynamicSmemBytes = sm;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_jacobi, a, J);
}

}  // namespace cupic
