// jacobi.cu -- Poisson solve (5-point Jacobi, periodic in x, Dirichlet in y)
// with the field derivation fused into the end of the last sweep
// (reference: jacobi_iteration mesh.cu:297-381, its host loop
// mesh.cu:55-120, field_derivation mesh.cu:385-472).
//
// The potential stays resident in shared memory for the whole solve: CTA c
// of a cooperative grid of G CTAs owns interior node rows [r0, r1) and keeps
// them, with K halo rows on each side, in two shared buffers (true Jacobi,
// not the reference's in-place update, defect D5).  Every K sweeps each CTA
// publishes its K first and K last rows to an L2-resident exchange buffer as
// words tagged with the exchange's epoch; a CTA waits only for its two
// neighbours' words.  Convergence checks use a grid barrier, and every wait
// is bounded: when a wait gives up the kernel raises CUPIC_FLAG_TIMEOUT and
// all CTAs return.
#include <math.h>

#include "cupic_internal.cuh"
#include "kernels.h"

namespace cupic {

namespace {

constexpr int kJBlock = 512;
constexpr long long kSpinLimit = 1ll << 22;
constexpr int kHaloBatch = 4;  // halo rows per side polled together
constexpr int kLoadBatch = 8;  // mesh values per thread loaded together at the start

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Halo words: a value and the epoch of the exchange that wrote it in one
// 64-bit word, written and read with single-copy-atomic relaxed accesses.
// A reader that sees the epoch it waits for has the value, so an exchange
// needs neither a fence nor a flag: one L2 round trip instead of three.
__device__ __forceinline__ void st_word(unsigned long long *p, float v, unsigned ep) {
  const unsigned long long w = ((unsigned long long)ep << 32) | __float_as_uint(v);
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(w) : "memory");
}
__device__ __forceinline__ unsigned long long ld_word(const unsigned long long *p) {
  unsigned long long w;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(w) : "l"(p) : "memory");
  return w;
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

// block max of non-negative doubles (their bit patterns order as unsigned
// 64-bit integers); every thread gets the result
__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long v,
                                                            unsigned long long *red) {
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = lane < (int)(blockDim.x >> 5) ? red[lane] : 0ull;
    for (int o = 16; o > 0; o >>= 1) w = max(w, __shfl_down_sync(0xffffffffu, w, o));
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

// The same sweep with each thread walking up a column: thread (gx, gy)
// computes the 4 nodes 4gx..4gx+3 of the consecutive rows [a0, a1), its
// share of [u0, u1) split into RPI near-equal segments.  The rows below and
// at the current one stay in registers from the previous step of the walk,
// so a row costs two 16-byte loads (the row above and the source) instead
// of four.  Every thread takes the same number of steps (the segment
// length), so the shuffles always see all 32 lanes; steps past a thread's
// segment compute from in-buffer rows and store nothing.
template <bool CHECK>
__device__ __forceinline__ float sweep_walk(const float *__restrict__ S, float *__restrict__ D,
                                            const float *__restrict__ bsrc, const SweepGeom &g, int u0,
                                            int u1, int o0, int o1) {
  const int P = g.P, W = g.W;
  const int n = u1 - u0;
  const int seg = (n + g.RPI - 1) / g.RPI;
  const int col = g.gx << 2;
  const bool lfix = g.lane == 0 || g.gx == 0;
  const bool rfix = g.lane == 31 || g.gx == g.TPR - 1;
  const bool seam = g.gx == 0;
  const int lcol = seam ? W - 1 : col - 1;
  const bool active = g.gy < g.RPI;
  const int a0 = u0 + (active ? g.gy : 0) * seg;
  const int a1 = active ? min(u1, a0 + seg) : a0;
  const int rs = a0 < u1 ? a0 : u0;  // first row read (in the buffer even for an empty segment)
  float4 sv = *reinterpret_cast<const float4 *>(S + (rs - 1) * P + col);
  float4 cv = *reinterpret_cast<const float4 *>(S + rs * P + col);
  float md = 0.0f;
  for (int t = 0; t < seg; ++t) {
    const int lr = a0 + t;
    const bool ok = lr < a1;
    const int lrc = ok ? lr : rs;
    const float *rowp = S + lrc * P;
    const float4 nv = *reinterpret_cast<const float4 *>(rowp + P + col);
    const float4 b4 = *reinterpret_cast<const float4 *>(bsrc + lrc * P + col);
    float lf = __shfl_up_sync(0xffffffffu, cv.w, 1);
    float rt = __shfl_down_sync(0xffffffffu, cv.x, 1);
    if (ok) {
      if (lfix) lf = rowp[lcol];
      if (rfix) rt = rowp[col + 4];  // col+4 == W is the seam copy of node 0
      float4 v;
      v.x = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(b4.x, lf), cv.y), nv.x), sv.x));
      v.y = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(b4.y, cv.x), cv.z), nv.y), sv.y));
      v.z = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(b4.z, cv.y), cv.w), nv.z), sv.z));
      v.w = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(b4.w, cv.z), rt), nv.w), sv.w));
      float *dp = D + lr * P;
      *reinterpret_cast<float4 *>(dp + col) = v;
      if (seam) dp[W] = v.x;
      if (CHECK && lr >= o0 && lr < o1) {
        md = fmaxf(md, fabsf(__fsub_rn(v.x, cv.x)));
        md = fmaxf(md, fabsf(__fsub_rn(v.y, cv.y)));
        md = fmaxf(md, fabsf(__fsub_rn(v.z, cv.z)));
        md = fmaxf(md, fabsf(__fsub_rn(v.w, cv.w)));
        if (seam) md = fmaxf(md, fabsf(__fsub_rn(v.x, rowp[W])));
      }
    }
    sv = cv;
    cv = nv;
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

// Register-strip sweep (used when (nnx-1) % 4 == 0 and the CTA's rows fit):
// thread (gx, gy) keeps the 4 nodes 4gx..4gx+3 of the R consecutive rows
// lr0 .. lr0+R-1 (lr0 = 1 + gy*R) in registers for the whole solve, with their
// source terms.  A sweep then reads from shared memory only the rows just
// below and above the strip and the west/east values at the ends of a warp
// or a row; the strip's own rows come from registers and its west/east
// neighbours by shuffle.  D receives only what other threads read: the
// strip's first and last rows (the neighbouring strips' south and north
// rows) and, of the rows between, the values at the ends of a warp's span
// and the seam columns -- every updated row in full only when `full` (the
// sweep before a halo exchange).  Halo rows outside the sweep's updated
// range [u0, u1) are computed too (sweep_reg says why no updated row ever
// reads them); the shared-memory path leaves them unwritten.
struct RegGeom {
  int P, W, NG, gx, gy, lane, lr0, nvalid, col, lcol;
  bool active, lfix, rfix, seam, whole_strip;
};

__device__ __forceinline__ float4 lds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

// FULL: the strip has all R rows (g.active and g.nvalid == R), known at
// compile time, so no row needs a select.
template <int R, bool CHECK, bool FULL = false>
__device__ __forceinline__ float sweep_reg(float4 (&x)[R], const float4 (&b)[R], const float *__restrict__ S,
                                           float *__restrict__ D, const RegGeom &g, int u0, int u1, int o0,
                                           int o1, bool full) {
  // Straight-line code over the strip's rows, so the rows' independent
  // chains can interleave: a row outside the strip computes from in-buffer
  // addresses (row 0) and its result is discarded by selects and predicated
  // stores.  Halo rows outside this sweep's updated range [u0, u1) are
  // computed like the others: by the temporal block's shrinking range, a
  // row outside it is read next only by rows outside the next sweep's
  // range, and the exchange at the end of the block replaces every halo
  // row (registers included), so their values never reach an updated row,
  // and the range test and its selects are spared.
  const int P = g.P, W = g.W, col = g.col;
  const bool any = g.active && g.nvalid > 0;
  const float4 s4 = lds4(S + (any ? g.lr0 - 1 : 0) * P + col);
  const float4 n4 = lds4(S + (any ? g.lr0 + g.nvalid : 0) * P + col);
  float4 prev = s4;
  float md = 0.0f;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const float4 c = x[r];
    float lf = __shfl_up_sync(0xffffffffu, c.w, 1);
    float rt = __shfl_down_sync(0xffffffffu, c.x, 1);
    const int lr = g.lr0 + r;
    const bool valid = FULL || (g.active && r < g.nvalid);
    const float *rowp = S + (valid ? lr : 0) * P;
    if (g.lfix) lf = rowp[g.lcol];
    if (g.rfix) rt = rowp[col + 4];
    const float4 nb = (r + 1 < R && (FULL || r + 1 < g.nvalid)) ? x[r + 1 < R ? r + 1 : r] : n4;
    float4 v;
    v.x = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(b[r].x, lf), c.y), nb.x), prev.x));
    v.y = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(b[r].y, c.x), c.z), nb.y), prev.y));
    v.z = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(b[r].z, c.y), c.w), nb.z), prev.z));
    v.w = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(b[r].w, c.z), rt), nb.w), prev.w));
    float *dp = D + (valid ? lr : 0) * P;
    const bool whole = full || r == 0 || r == (FULL ? R : g.nvalid) - 1;
    if (valid && whole) *reinterpret_cast<float4 *>(dp + col) = v;
    if (valid && !whole && g.lfix) dp[col] = v.x;      // east neighbour of the lane before
    if (valid && !whole && g.rfix) dp[col + 3] = v.w;  // west neighbour of the lane after (or of column 0)
    if (valid && g.seam) dp[W] = v.x;
    if (CHECK && valid && lr >= o0 && lr < o1) {
      md = fmaxf(md, fabsf(__fsub_rn(v.x, c.x)));
      md = fmaxf(md, fabsf(__fsub_rn(v.y, c.y)));
      md = fmaxf(md, fabsf(__fsub_rn(v.z, c.z)));
      md = fmaxf(md, fabsf(__fsub_rn(v.w, c.w)));
      if (g.seam) md = fmaxf(md, fabsf(__fsub_rn(v.x, rowp[W])));
    }
    x[r] = valid ? v : c;
    prev = c;  // the previous value of row r is the south neighbour of row r+1
  }
  return md;
}

// Rows of CTA c: interior rows [r0, r1) with r0 = 1 + c*M/G (M = nny-2), so
// every CTA owns floor(M/G) or ceil(M/G) rows.  With temporal blocking depth
// k, a CTA also holds k halo rows on each side; sweep m (1..k) after an
// exchange updates the rows [r0-k+m, r1+k-m) -- the halo part redundantly,
// with the same operands as the neighbour, so the values are identical --
// and the neighbours trade their k boundary rows only every k sweeps.
// R > 0 selects the register-strip sweep with strips of R rows; R == 0 the
// shared-memory sweep (sweep_walk / sweep_vec / sweep_scalar).
// the kernels' static shared scratch, one copy for every sweep form
struct JScratch {
  float red[33];                 // block_max
  unsigned long long red64[33];  // block_max_u64
  int bail;
};

template <int R>
__device__ __forceinline__ void jacobi_body(const SimArgs &a, const JacobiArgs &J, const int c, float *jsm,
                                            JScratch *js) {
  int &bail = js->bail;
  float *const red = js->red;
  // uniform: flags of earlier kernels
  if (halted(a.ctl) || (J.gated && *reinterpret_cast<volatile int *>(&a.ctl->refine_done))) return;
  const int G = J.G, tid = threadIdx.x;
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

  float *const phi = J.phi ? J.phi : a.phi;
  const long long *acc = reinterpret_cast<const long long *>(a.rho[ctl->cur]);
  // epochs of this solve's exchanges e = 1, 2, ...: (solve count << 16) + e,
  // never 0 (the cleared buffer) and never those of an earlier solve's
  // words still in the buffer
  const unsigned ebase = *reinterpret_cast<volatile unsigned *>(&ctl->jepoch) << 16;
  if (J.zero_next) {
    // the accumulator the step's push deposits into: this CTA's rows, and
    // the boundary rows from the first and last CTA
    unsigned long long *nx = a.rho[ctl->cur ^ 1];
    const int z0 = c == 0 ? 0 : r0, z1 = c == G - 1 ? nny : r1;
    for (size_t k = (size_t)z0 * nnx + tid; k < (size_t)z1 * nnx; k += kJBlock) nx[k] = 0ull;
  }
  // Load the buffered rows: the (row, column) pairs taken kLoadBatch at a
  // time per thread with all their loads issued before the first store, so
  // a batch costs one memory round trip instead of one per row.  A fused
  // correction forms its source here: the FP64 residual of the node, in the
  // operation order of k_r64_residual (refine.cu), rounded to FP32 once; the
  // max |r| over the CTA's owned rows feeds the stop test.
  double rmax = 0.0;
  {
    const int total = nrows * nnx;
    for (int k0 = tid; k0 < total; k0 += kJBlock * kLoadBatch) {
      float v[kLoadBatch], bv[kLoadBatch];
#pragma unroll
      for (int u = 0; u < kLoadBatch; ++u) {
        const int k = k0 + u * kJBlock;
        v[u] = 0.0f;
        bv[u] = 0.0f;
        if (k < total) {
          const int lr = k / nnx, i = k - lr * nnx, j = lo + lr;
          const size_t rb = (size_t)j * nnx;
          v[u] = J.phi_zero ? 0.0f : phi[rb + i];
          if (j >= 1 && j <= nny - 2) {
            if (J.r64_phi) {
              const double *q = J.r64_phi;
              const int ii = i == nnx - 1 ? 0 : i;  // the mirror column carries column 0's residual
              const double cc = q[rb + ii];
              const double w = q[rb + (ii == 0 ? nnx - 2 : ii - 1)];
              const double e = q[rb + ii + 1];
              const double n = q[rb + nnx + ii], so = q[rb - nnx + ii];
              const double r = J.r64_b[rb + ii] - (4.0 * cc - (((w + e) + n) + so));
              bv[u] = __double2float_rn(r);
              if (j >= r0 && j < r1) rmax = fmax(rmax, fabs(r));
            } else if (J.src) {
              bv[u] = J.src[rb + i];
            } else {
              const long long f = (i == 0 || i == nnx - 1) ? acc[rb] + acc[rb + nnx - 1] : acc[rb + i];
              bv[u] = __double2float_rn((double)f * a.cb);
            }
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kLoadBatch; ++u) {
        const int k = k0 + u * kJBlock;
        if (k < total) {
          const int lr = k / nnx, i = k - lr * nnx, j = lo + lr;
          buf0[lr * P + i] = v[u];
          buf1[lr * P + i] = v[u];
          if (j >= 1 && j <= nny - 2) bsrc[lr * P + i] = bv[u];
        }
      }
    }
  }
  __syncthreads();

  // a fused correction: the stop test of the solve on the grid's max |r|
  int chk0 = 0;  // rounds of the grid barrier counter used so far
  if (J.r64_phi) {
    unsigned long long *const red64 = js->red64;
    unsigned long long gm = block_max_u64((unsigned long long)__double_as_longlong(rmax), red64);
    if (G > 1) {
      // the CTAs' maxima in the residual slots, read back after a grid
      // barrier (a fused correction runs no convergence checks, which use
      // the same slots)
      unsigned long long *slots = reinterpret_cast<unsigned long long *>(J.res_cta);
      if (tid == 0) {
        __stcg(&slots[c], gm);
        __threadfence();
        atomicAdd(J.bar, 1u);
        if (!wait_geq(J.bar, (unsigned)G, ctl)) bail = 1;
      }
      __syncthreads();
      if (bail) return;
      unsigned long long m = 0ull;
      for (int k = tid; k < G; k += kJBlock) m = max(m, __ldcg(&slots[k]));
      gm = block_max_u64(m, red64);
      chk0 = 1;
    }
    const double res = __longlong_as_double((long long)gm);
    if ((J.r64_done >= J.r64_mn && res < J.r64_tol) || J.r64_done >= J.r64_mx) {
      if (c == 0 && tid == 0) {
        ctl->refine_done = 1;
        if (J.r64_stats) {
          ctl->sweeps = J.r64_done;
          ctl->residual = (float)res;
        }
      }
      return;  // no sweeps, so no halo words of this solve's epochs
    }
  }

  const int W = nnx - 1;  // computed columns 0 .. nnx-2; column nnx-1 mirrors 0
  const int o0 = r0 - lo, o1 = r1 - lo;  // owned local rows
  // shared-memory sweep geometry (R == 0)
  const bool vec = J.vec != 0;
  SweepGeom sg;
  sg.P = P;
  sg.W = W;
  sg.NG = vec ? (W >> 2) : W;
  sg.TPR = min(sg.NG, kJBlock);
  sg.RPI = kJBlock / sg.TPR;
  sg.gx = tid % sg.TPR;
  sg.gy = tid / sg.TPR;
  sg.lane = tid & 31;
  // register-strip geometry (R > 0)
  RegGeom rg;
  float4 x[R > 0 ? R : 1], bb[R > 0 ? R : 1];
  if (R > 0) {
    rg.P = P;
    rg.W = W;
    rg.NG = W >> 2;
    rg.gx = tid % rg.NG;
    rg.gy = tid / rg.NG;
    rg.lane = tid & 31;
    rg.lr0 = 1 + rg.gy * R;
    rg.active = rg.lr0 < nrows - 1;
    rg.nvalid = rg.active ? min(R, nrows - 1 - rg.lr0) : 0;
    // the same for every lane of a warp (its sweep shuffles across all 32):
    // a warp whose lanes hold strips of different lengths takes the
    // general form
    rg.whole_strip = __all_sync(0xffffffffu, rg.active && rg.nvalid == R);
    rg.col = rg.gx << 2;
    rg.seam = rg.gx == 0;
    rg.lcol = rg.seam ? W - 1 : rg.col - 1;
    rg.lfix = rg.lane == 0 || rg.gx == 0;
    rg.rfix = rg.lane == 31 || rg.gx == rg.NG - 1;
#pragma unroll
    for (int r = 0; r < (R > 0 ? R : 1); ++r) {
      x[r] = make_float4(0.f, 0.f, 0.f, 0.f);
      bb[r] = x[r];
      if (r < rg.nvalid) {
        x[r] = lds4(buf0 + (rg.lr0 + r) * P + rg.col);
        bb[r] = lds4(bsrc + (rg.lr0 + r) * P + rg.col);
      }
    }
  }
  auto sweep = [&](const float *S, float *D, int u0, int u1, bool check, bool full) -> float {
    if constexpr (R > 0) {
      if (check) return sweep_reg<R, true>(x, bb, S, D, rg, u0, u1, o0, o1, full);
      return rg.whole_strip ? sweep_reg<R, false, true>(x, bb, S, D, rg, u0, u1, o0, o1, full)
                            : sweep_reg<R, false>(x, bb, S, D, rg, u0, u1, o0, o1, full);
    } else {
      if (u0 >= u1) return 0.0f;
      // long segments walk up the columns; short ones (a few rows per
      // thread, where the walk's serial steps cost more than its loads
      // save) take the rows in turn
      if (vec && u1 - u0 >= 4 * sg.RPI)
        return check ? sweep_walk<true>(S, D, bsrc, sg, u0, u1, o0, o1)
                     : sweep_walk<false>(S, D, bsrc, sg, u0, u1, o0, o1);
      if (vec) return check ? sweep_vec<true>(S, D, bsrc, sg, u0, u1, o0, o1)
                            : sweep_vec<false>(S, D, bsrc, sg, u0, u1, o0, o1);
      return check ? sweep_scalar<true>(S, D, bsrc, sg, u0, u1, o0, o1)
                   : sweep_scalar<false>(S, D, bsrc, sg, u0, u1, o0, o1);
    }
  };
  // Halo exchange.  Each CTA writes its K first and K last rows as halo
  // words of the exchange's epoch; the neighbours poll the words they need
  // until every one carries that epoch.  The slots alternate by the
  // exchange's parity: a CTA overwrites a slot two exchanges later, after
  // its neighbours' next words, and so their reads of this one, arrived.
  auto publish = [&](const float *D, int e) {
    const unsigned ep = ebase + (unsigned)e;
    unsigned long long *hp = J.halo + ((size_t)(e & 1) * G + c) * 2 * K * P;
    for (int i = tid; i < nnx; i += kJBlock) {
      for (int r = 0; r < K; ++r) {
        st_word(hp + r * P + i, D[(o0 + r) * P + i], ep);
        st_word(hp + (K + r) * P + i, D[(o1 - K + r) * P + i], ep);
      }
    }
  };
  auto receive = [&](float *D, int e) -> bool {
    const unsigned ep = ebase + (unsigned)e;
    const unsigned long long *hlo = J.halo + ((size_t)(e & 1) * G + (c - 1)) * 2 * K * P + K * P;
    const unsigned long long *hhi = J.halo + ((size_t)(e & 1) * G + (c + 1)) * 2 * K * P;
    bool ok = true;
    // A thread takes columns i and i + kJBlock together, all their loads in
    // flight at once: with one column per pass, the thread that also held
    // column 512 of a 513-node row polled twice in series, and every CTA
    // waited for its second L2 round trip at every exchange.
    const unsigned long long none = (unsigned long long)ep << 32;  // a word needing no wait
    for (int i = tid; i < nnx && ok; i += 2 * kJBlock) {
      const int i2 = i + kJBlock;
      const bool two = i2 < nnx;
      for (int rb = 0; rb < K && ok; rb += kHaloBatch) {  // batches of rows per side, all loads in flight
        unsigned long long wl[kHaloBatch], wh[kHaloBatch], wl2[kHaloBatch], wh2[kHaloBatch];
        for (long long it = 0;; ++it) {
          bool all = true;
#pragma unroll
          for (int q = 0; q < kHaloBatch; ++q) {
            const int r = rb + q;
            const bool lo_ok = r < K && c > 0, hi_ok = r < K && c < G - 1;
            wl[q] = lo_ok ? ld_word(hlo + r * P + i) : none;
            wh[q] = hi_ok ? ld_word(hhi + r * P + i) : none;
            wl2[q] = (two && lo_ok) ? ld_word(hlo + r * P + i2) : none;
            wh2[q] = (two && hi_ok) ? ld_word(hhi + r * P + i2) : none;
          }
#pragma unroll
          for (int q = 0; q < kHaloBatch; ++q)
            all = all && (unsigned)(wl[q] >> 32) == ep && (unsigned)(wh[q] >> 32) == ep &&
                  (unsigned)(wl2[q] >> 32) == ep && (unsigned)(wh2[q] >> 32) == ep;
          if (all) break;
          if (it >= kSpinLimit || ((it & 255) == 255 && *(volatile int *)&ctl->abort)) {
            ok = false;
            break;
          }
          if (it > 4096) __nanosleep(32);
        }
        if (!ok) break;
#pragma unroll
        for (int q = 0; q < kHaloBatch; ++q) {
          const int r = rb + q;
          // the lower neighbour's last K rows, the upper neighbour's first K rows
          if (r < K && c > 0) {
            D[(o0 - K + r) * P + i] = __uint_as_float((unsigned)wl[q]);
            if (two) D[(o0 - K + r) * P + i2] = __uint_as_float((unsigned)wl2[q]);
          }
          if (r < K && c < G - 1) {
            D[(o1 + r) * P + i] = __uint_as_float((unsigned)wh[q]);
            if (two) D[(o1 + r) * P + i2] = __uint_as_float((unsigned)wh2[q]);
          }
        }
      }
    }
    if (!ok) {
      if (!*(volatile int *)&ctl->abort) {
        atomicExch(&ctl->abort, 1);
        atomicOr(&ctl->step_flags, (uint32_t)CUPIC_FLAG_TIMEOUT);
      }
      bail = 1;
    }
    __syncthreads();
    if (bail) return false;
    if constexpr (R > 0) {  // the strips' halo rows are new: reload their registers
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int lr = rg.lr0 + r;
        if (r < rg.nvalid && (lr < o0 || lr >= o1)) x[r] = lds4(D + lr * P + rg.col);
      }
    }
    return true;
  };

  int src = 0, done = 0, nchk = chk0, m = 0, pending = 0, to_check = J.check_every;
  float last = INFINITY;
  for (int s = 1; s <= J.max_sweeps; ++s) {
    float *S = src ? buf1 : buf0;
    float *D = src ? buf0 : buf1;
    // a solve with no tolerance that reports nothing (a correction of the
    // precision form) needs no residual: no check, no grid barrier.  A
    // check before min_sweeps can stop nothing, and a later check replaces
    // its residual, so those are skipped: a fixed-sweep solve (min = max)
    // checks once, after its last sweep, with the same result and report.
    const bool due = --to_check == 0;
    if (due) to_check = J.check_every;
    const bool check = ((due && s >= J.min_sweeps) || s == J.max_sweeps) && (J.tol > 0.0 || J.write_stats);
    m = (m >= K) ? 1 : m + 1;                        // position in the temporal block
    const int u0 = max(1, r0 - K + m) - lo;          // updated local rows [u0, u1)
    const int u1 = min(nny - 2, r1 - 1 + K - m) + 1 - lo;
    const bool full = G > 1 && m == K;  // a halo exchange follows this sweep
    float md;
    if (R > 0) {
      if (pending) {
        if (!receive(S, pending)) break;
        pending = 0;
      }
      md = sweep(S, D, u0, u1, check, full);
    } else if (pending) {
      // rows o0+1 .. o1-2 read only owned rows of S: sweep them first
      const int i0 = max(u0, o0 + 1), i1 = min(u1, o1 - 1);
      md = sweep(S, D, i0, i1, check, full);
      if (!receive(S, pending)) break;
      md = fmaxf(md, sweep(S, D, u0, min(i0, u1), check, full));
      md = fmaxf(md, sweep(S, D, max(i1, u0), u1, check, full));
      pending = 0;
    } else {
      md = sweep(S, D, u0, u1, check, full);
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
  if constexpr (R > 0) {
    // the strips' rows in full: the rows between a strip's first and last
    // are current only in registers
    if (rg.active) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (r < rg.nvalid) {
          float *dp = F + (rg.lr0 + r) * P;
          *reinterpret_cast<float4 *>(dp + rg.col) = x[r];
          if (rg.seam) dp[rg.W] = x[r].x;
        }
      }
    }
    __syncthreads();
  }

  // write back the owned rows; derive E = -grad phi (mesh.cu:413-468).  The
  // rows r0-1 and r1 are current: either just exchanged or updated in the
  // last sweep of an unfinished temporal block.
  if (J.r64_phi) {
    // a fused correction: phi64 += correction on the owned rows (every
    // column, the mirror included, as k_r64_update does)
    if (done > 0)
      for (int lr = o0; lr < o1; ++lr)
        for (int i = tid; i < nnx; i += kJBlock)
          J.r64_phi[(size_t)(lo + lr) * nnx + i] += (double)F[lr * P + i];
  } else {
    for (int lr = o0; lr < o1; ++lr)
      for (int i = tid; i < nnx; i += kJBlock) phi[(size_t)(lo + lr) * nnx + i] = F[lr * P + i];
  }
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
  // the next solve's epochs: the last CTA to finish advances the base, when
  // every CTA of this solve has read it (each reads it first thing)
  if (tid == 0) {
    __threadfence();
    if (atomicAdd(&ctl->jdone, 1u) == (unsigned)G - 1u) {
      ctl->jdone = 0u;
      atomicAdd(&ctl->jepoch, 1u);
    }
  }
}

__device__ __forceinline__ void jacobi_dispatch(const SimArgs &a, const JacobiArgs &J, int c, float *jsm,
                                                JScratch *js) {
  switch (J.strip) {
    case 1: jacobi_body<1>(a, J, c, jsm, js); break;
    case 2: jacobi_body<2>(a, J, c, jsm, js); break;
    case 3: jacobi_body<3>(a, J, c, jsm, js); break;
    case 4: jacobi_body<4>(a, J, c, jsm, js); break;
    case 5: jacobi_body<5>(a, J, c, jsm, js); break;
    case 6: jacobi_body<6>(a, J, c, jsm, js); break;
    case 7: jacobi_body<7>(a, J, c, jsm, js); break;
    case 8: jacobi_body<8>(a, J, c, jsm, js); break;
    default: jacobi_body<0>(a, J, c, jsm, js); break;
  }
}

__global__ void __launch_bounds__(kJBlock, 1) k_jacobi(SimArgs a, JacobiArgs J) {
  extern __shared__ __align__(16) float jsm[];
  __shared__ JScratch js;
  if (threadIdx.x == 0) js.bail = 0;
  __syncthreads();
  jacobi_dispatch(a, J, blockIdx.x, jsm, &js);
}

// Many contexts' solves in one cooperative launch.  The grid is split into
// groups of CTAs; group g (CTAs first .. first+G-1) solves the instances
// list[begin .. end) one after another, its CTA c acting as CTA c of each
// solve.  The instances of a group share its CTA count; their exchange
// flags are zeroed before the launch.
__global__ void __launch_bounds__(kJBlock, 1)
    k_jacobi_batch(const SimArgs *__restrict__ inst, const JacobiArgs *__restrict__ jargs,
                   const JGroup *__restrict__ groups, int ngroups, const int *__restrict__ list) {
  extern __shared__ __align__(16) float jsm[];
  __shared__ JScratch js;
  int g = 0;
  while (g + 1 < ngroups && groups[g + 1].first <= (int)blockIdx.x) ++g;
  const JGroup gr = groups[g];
  const int c = (int)blockIdx.x - gr.first;
  if (c < 0 || c >= gr.G) return;
  for (int q = gr.begin; q < gr.end; ++q) {
    const int i = list[q];
    if (threadIdx.x == 0) js.bail = 0;
    __syncthreads();
    jacobi_dispatch(inst[i], jargs[i], c, jsm, &js);
    __syncthreads();
  }
}

// strip height for the register-strip sweep: the smallest R in 1..8 whose
// strips cover `urows` updatable rows of (nnx-1)/4 column groups with one
// thread each; 0 (shared-memory sweep) when none does.  Every height, not
// only powers of two: at 512x2048 (152 CTAs of 14 rows, halo depth 4) the
// 20 rows take R = 5 on all 512 threads, where R = 8 left a quarter of them
// idle; the solve went from 0.399 to 0.385 ms.
int jacobi_strip_rows(int nnx, int urows) {
  if ((nnx - 1) % 4 != 0) return 0;
  const int ng = (nnx - 1) / 4;
  if (ng > kJBlock) return 0;
  for (int r = 1; r <= 8; ++r)
    if ((long long)ng * ((urows + r - 1) / r) <= kJBlock) return r;
  return 0;
}

size_t jacobi_smem_bytes(int rows_per_cta, int depth, int pitch) {
  return (size_t)3 * (rows_per_cta + 2 * depth) * pitch * sizeof(float);
}

cudaError_t jacobi_set_smem(size_t bytes) {
  return raise_dyn_smem(reinterpret_cast<const void *>(k_jacobi), bytes);
}

cudaError_t jacobi_max_ctas(size_t smem, int *per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_jacobi, kJBlock, smem);
}

// Fault-detection self-test: one thread waits, through the solver's bounded
// wait, on a word of the control block that nothing writes.  The wait gives
// up after its iteration limit and raises CUPIC_FLAG_TIMEOUT.
__global__ void k_wait_probe(SimArgs a) {
  if (threadIdx.x == 0) wait_geq(&a.ctl->idle, 1u, a.ctl);
}

cudaError_t launch_wait_probe(const SimArgs &a, cudaStream_t st) {
  k_wait_probe<<<1, 32, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t jacobi_batch_set_smem(size_t bytes) {
  return raise_dyn_smem(reinterpret_cast<const void *>(k_jacobi_batch), bytes);
}

cudaError_t jacobi_batch_max_ctas(size_t smem, int *per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_jacobi_batch, kJBlock, smem);
}

cudaError_t launch_jacobi_batch(const SimArgs *inst, const JacobiArgs *jargs, const JGroup *groups,
                                int ngroups, const int *list, int nctas, size_t smem, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nctas);
  cfg.blockDim = dim3(kJBlock);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_jacobi_batch, inst, jargs, groups, ngroups, list);
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
