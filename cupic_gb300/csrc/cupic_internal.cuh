// cupic_internal.cuh -- device-side state layout and per-particle arithmetic
// of the GB300 PIC cycle.  Every floating-point operation here rounds where
// the source says: the library is compiled with -fmad=false and uses
// explicit __fmaf_rn / __fma_rn where a fused multiply-add is intended, so
// the CPU oracle can reproduce each result bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/cupic_gpu.h"

namespace cupic {

constexpr int kRowAbsorbed = -1;
constexpr int kRowRemoved = -2;
constexpr int kStatsRing = 4096;      // per-step stats kept on the device
constexpr int kPurposeInit = 0;       // Philox counter word 3, bits 8..15
constexpr int kPurposeInject = 1;

// Control block resident in device memory; the kernels of a step read and
// advance it, so a captured graph of one step can be replayed unchanged.
struct Ctl {
  int64_t step;           // index i of the next step (main.cu:59)
  double t;               // time passed to the boundary stage of that step
  double tin[2];          // next injection time per species (cc.cu:35-36)
  int32_t tin_set[2];     // 0 until the first boundary call
  int32_t cur;            // rho[cur] holds the charge of the current particles
  uint32_t flags;         // sticky CUPIC_FLAG_* bits
  uint32_t step_flags;    // flags raised during the current step
  int32_t sweeps;         // Jacobi sweeps of the last solve
  float residual;         // max |dphi| of its last checked sweep
  int32_t inj_count[2];   // injected this step
  int32_t inj_gen[2];     // draws generated this step (inj_count capped at inj_cap)
  unsigned long long absorbed[2];
  unsigned long long removed[2];
  int32_t abort;          // a bounded wait gave up: kernels bail out
  int32_t halt;           // a row cannot take the step's arrivals: the rest of the run is idle
  int32_t skipped;        // steps whose bookkeeping found the run halted (the halted one included)
  uint32_t jepoch;        // solves run so far: the base of the halo words' epochs
  uint32_t idle;          // never written: the bounded-wait self-test waits on it
  int32_t refine_done;    // precision-form solve: the stop test passed, later corrections idle
  uint32_t jdone;         // CTAs of the running solve that have finished (the last one resets it)
  uint32_t pad;
  cupic_step_stats ring[kStatsRing];
};

// Per-species particle storage: rows are contiguous segments of `parts`
// with fixed capacity; the live prefix of row j is [seg[j], seg[j]+cnt[j]).
struct SpeciesDev {
  float4 *parts;          // {x, y, vx, vy}
  int64_t *seg;           // [ncy] segment start
  int32_t *cap;           // [ncy] segment capacity
  int32_t *cnt;           // [ncy] live particles
  int32_t *nstay;         // [ncy] stayed in the row this step
  int32_t *nup;           // [ncy] moved to row+1 (staged in stage_up)
  int32_t *ndown;         // [ncy] moved to row-1 (staged in stage_down)
  float4 *stage_up;       // [ncy * stage_cap]
  float4 *stage_down;     // [ncy * stage_cap]
  int32_t stage_cap;
  int32_t inj_cap;        // most particles injected per step
  double *inj_tin;        // [inj_cap] scratch: injection time of each draw
  float4 *inj_p;          // [inj_cap] scratch: the injected particles of the step
  int32_t *inj_d;         // [inj_cap] scratch: their rows (< 0: removed)
};

// Everything a kernel needs, passed by value.
struct SimArgs {
  int ncx, ncy, nnx, nny;
  // single-precision constants, each rounded once from double
  float ds, inv_ds, Lx, Ly, two_ds, dt;
  float dtqm[2], mhdtqm[2];
  // double-precision constants (injection, charge conversion)
  double ds_d, inv_ds_d, Lx_d, Ly_d, dt_d;
  double cb;              // fixed-point charge -> Jacobi source term
  double dtin[2], qm[2], sig[2];
  int32_t ppr;
  uint32_t k0, k1;        // generator key (seed)
  SpeciesDev sp[2];
  float *phi;             // [nny*nnx]
  float2 *E;              // [nny*nnx] {Ex, Ey}
  unsigned long long *rho[2];  // raw (unfolded) fixed-point charge, 2^32 per unit
  Ctl *ctl;
};

// Jacobi launch description (see jacobi.cu).
struct JacobiArgs {
  double tol;
  int32_t min_sweeps, max_sweeps, check_every;
  int32_t G;              // CTAs (cooperative)
  int32_t rows_per_cta;   // most interior rows owned by one CTA: ceil((nny-2)/G)
  int32_t depth;          // temporal blocking: sweeps between halo exchanges (G > 1)
  int32_t pitch;          // smem row pitch in floats (a multiple of 4)
  int32_t vec;            // 1: (nnx-1) % 4 == 0, sweep 4 nodes per thread with float4
  int32_t strip;          // 0: shared-memory sweep; 1, 2, 4, 8: rows kept in registers per thread
  int32_t do_field;       // 1: derive E after the last sweep
  int32_t write_stats;    // 1: store sweeps/residual in the control block
  int32_t zero_next;      // 1: also clear the next charge accumulator a.rho[cur^1] (a step's solve)
  int32_t gated;          // 1: return at once when ctl->refine_done is set (precision-form correction)
  int32_t phi_zero;       // 1: the initial potential is zero everywhere and is not read
  unsigned int *flags;    // [G] last sweep published by each CTA
  unsigned int *bar;      // [1] grid barrier counter
  float *res_cta;         // [2*G] per-CTA max |dphi| of a checked sweep
  unsigned long long *halo;  // [2 parity][G][2 sides][depth rows][pitch] {value, epoch} words
  float *phi;             // the potential solved for; NULL: a.phi
  const float *src;       // FP32 source per node; NULL: the charge accumulator a.rho[cur]
  // A correction of the precision form with its residual, stop test and
  // update fused in (r64_phi != NULL; phi is the correction, phi_zero set,
  // no convergence checks): the kernel forms the FP64 residual
  // r = b - A phi64 of its rows as its FP32 source, takes the max norm over
  // the grid, and applies the stop test of the solve (after r64_done
  // correction sweeps: stop when r64_done >= r64_mn and max |r| < r64_tol,
  // or r64_done >= r64_mx; the stopping test sets ctl->refine_done and, with
  // r64_stats, records the sweeps and the residual).  If it goes on, it runs
  // its sweeps and adds the correction to phi64 on its owned rows.
  double *r64_phi;
  const double *r64_b;
  double r64_tol;
  int32_t r64_done, r64_mn, r64_mx, r64_stats;
};

// a group of CTAs of the batched solve and its instances (list[begin..end))
struct JGroup {
  int32_t first, G, begin, end;
};

// Set by the room check of a step whose arrivals do not fit their rows; the
// host grows those rows and completes the step.  Every kernel of a step
// reads it first and returns when it is set: the flag changes only between
// kernels, so the whole grid sees one value.
__device__ __forceinline__ bool halted(const Ctl *ctl) {
  return *reinterpret_cast<const volatile int32_t *>(&ctl->halt) != 0;
}

// ---------------------------------------------------------------------------
// arithmetic shared by the kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ float clamp01f(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }
__device__ __forceinline__ double clamp01d(double v) { return fmin(fmax(v, 0.0), 1.0); }

// floor(v) clamped to [0, hi]; NaN -> 0.  cvt.rmi saturates out-of-range
// values and maps NaN to 0, so one conversion and an integer clamp give the
// same result as the oracle's explicit tests.
__device__ __forceinline__ int cfloorf(float v, int lo, int hi) {
  return min(max(__float2int_rd(v), lo), hi);
}
__device__ __forceinline__ int cfloord(double v, int lo, int hi) {
  if (!(v >= (double)lo)) return lo;
  if (v >= (double)(hi + 1)) return hi;
  int i = (int)floor(v);
  return i > hi ? hi : i;
}

// Floor and nearest-even rounding of floats in [-0, 2^23) on the FP32 pipe
// instead of the conversion unit: t = v + 2^23 rounded down (or to nearest
// even) is exactly 2^23 + floor(v) (or rint(v)), whose bits less those of
// 2^23 are that integer; 2^23 - t rounded down is minus it as a float,
// exactly, with -0 for 0 (as -(float)0).
constexpr float kMagic23 = 8388608.0f;
constexpr int kMagic23Bits = 0x4B000000;
__device__ __forceinline__ int magic_int(float t) { return __float_as_int(t) - kMagic23Bits; }
__device__ __forceinline__ float neg_magic_float(float t) { return __fsub_rd(kMagic23, t); }

__device__ __forceinline__ int row_of(const SimArgs &a, float y) {
  return cfloorf(__fmul_rn(y, a.inv_ds), 0, a.ncy - 1);
}

// periodic x: [0, Lx), applied as two sequential tests so that a tiny
// negative x that rounds to Lx after +Lx ends at 0
__device__ __forceinline__ float wrap_x(const SimArgs &a, float x) {
  if (x < 0.0f) x = __fadd_rn(x, a.Lx);
  if (x >= a.Lx) x = __fsub_rn(x, a.Lx);
  return x;
}

// Philox4x32-10 (Salmon et al., SC'11)
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

__device__ __forceinline__ double u01(uint32_t r) { return ((double)r + 0.5) * 0x1p-32; }

// natural log from IEEE basic operations (exponent split, atanh series)
__device__ __forceinline__ double dev_log(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  int e = (int)((b >> 52) & 0x7ff) - 1023;
  b = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull;
  double m = __longlong_as_double((long long)b);
  if (m > 1.4142135623730951) {
    m = m * 0.5;
    e += 1;
  }
  const double s = (m - 1.0) / (m + 1.0);
  const double s2 = s * s;
  double q = 1.0 / 23.0;
  q = q * s2 + 1.0 / 21.0;
  q = q * s2 + 1.0 / 19.0;
  q = q * s2 + 1.0 / 17.0;
  q = q * s2 + 1.0 / 15.0;
  q = q * s2 + 1.0 / 13.0;
  q = q * s2 + 1.0 / 11.0;
  q = q * s2 + 1.0 / 9.0;
  q = q * s2 + 1.0 / 7.0;
  q = q * s2 + 1.0 / 5.0;
  q = q * s2 + 1.0 / 3.0;
  q = q * s2 + 1.0;
  return (double)e * 0.69314718055994531 + 2.0 * s * q;
}

// sin, cos of th in [0, pi/4], Taylor series to th^17 / th^16
__device__ __forceinline__ void dev_sincos_small(double th, double *s, double *c) {
  const double t2 = th * th;
  double ps = -1.0 / 355687428096000.0;
  ps = ps * t2 + 1.0 / 1307674368000.0;
  ps = ps * t2 - 1.0 / 6227020800.0;
  ps = ps * t2 + 1.0 / 39916800.0;
  ps = ps * t2 - 1.0 / 362880.0;
  ps = ps * t2 + 1.0 / 5040.0;
  ps = ps * t2 - 1.0 / 120.0;
  ps = ps * t2 + 1.0 / 6.0;
  *s = th - th * t2 * ps;
  double pc = 1.0 / 20922789888000.0;
  pc = pc * t2 - 1.0 / 87178291200.0;
  pc = pc * t2 + 1.0 / 479001600.0;
  pc = pc * t2 - 1.0 / 3628800.0;
  pc = pc * t2 + 1.0 / 40320.0;
  pc = pc * t2 - 1.0 / 720.0;
  pc = pc * t2 + 1.0 / 24.0;
  pc = pc * t2 - 0.5;
  *c = 1.0 + t2 * pc;
}

// sin(2 pi u), cos(2 pi u), u in [0,1), by octant reduction
__device__ __forceinline__ void dev_sincos2pi(double u, double *s, double *c) {
  const double r = u * 8.0;
  int o = (int)r;
  o = o > 7 ? 7 : (o < 0 ? 0 : o);
  const double f = r - (double)o;
  const double qpi = 0.78539816339744831;
  double sa, ca;
  dev_sincos_small(((o & 1) ? (1.0 - f) : f) * qpi, &sa, &ca);
  switch (o) {
    case 0: *s = sa; *c = ca; break;
    case 1: *s = ca; *c = sa; break;
    case 2: *s = ca; *c = -sa; break;
    case 3: *s = sa; *c = -ca; break;
    case 4: *s = -sa; *c = -ca; break;
    case 5: *s = -ca; *c = -sa; break;
    case 6: *s = -ca; *c = sa; break;
    default: *s = -sa; *c = ca; break;
  }
}

// CIC field at a particle of cell row s, from a shared tile holding node
// rows s and s+1 (tile row stride = nnx).
__device__ __forceinline__ void gather_tile(const SimArgs &a, const float2 *tile, float x, float y,
                                            int s, float &Epx, float &Epy) {
  // x and y components side by side in packed FP32x2 operations; each
  // component is rounded exactly as its scalar operation
  const float2 sxy = __fmul2_rn(make_float2(x, y), make_float2(a.inv_ds, a.inv_ds));
  const int ic = cfloorf(sxy.x, 0, a.ncx - 1);
  const float2 d = __fadd2_rn(sxy, make_float2(-(float)ic, -(float)s));  // sx - ic, sy - s
  const float fx = clamp01f(d.x), fy = clamp01f(d.y);
  const float2 g = __fadd2_rn(make_float2(1.0f, 1.0f), make_float2(-fx, -fy));  // gx, gy
  const float2 wlo = __fmul2_rn(make_float2(g.x, fx), make_float2(g.y, g.y));    // w00, w10
  const float2 whi = __fmul2_rn(make_float2(g.x, fx), make_float2(fy, fy));      // w01, w11
  const float2 e00 = tile[ic], e10 = tile[ic + 1];
  const float2 e01 = tile[a.nnx + ic], e11 = tile[a.nnx + ic + 1];
  float2 e = __fmul2_rn(make_float2(wlo.x, wlo.x), e00);
  e = __ffma2_rn(make_float2(wlo.y, wlo.y), e10, e);
  e = __ffma2_rn(make_float2(whi.x, whi.x), e01, e);
  e = __ffma2_rn(make_float2(whi.y, whi.y), e11, e);
  Epx = e.x;
  Epy = e.y;
}

// The same gather from a tile of node pairs: entry i of a row holds nodes
// i and i+1 of that row as {Ex_i, Ey_i, Ex_i+1, Ey_i+1}, rows of nnx-1
// entries, so a particle reads its four nodes with two 16-byte loads.  The
// values and the order of operations are those of gather_tile.
__device__ __forceinline__ void gather_pairs(const SimArgs &a, const float4 *tile, float x, float y,
                                             int s, float &Epx, float &Epy) {
  const float2 sxy = __fmul2_rn(make_float2(x, y), make_float2(a.inv_ds, a.inv_ds));
  // ic = floor(sx) clamped to [0, ncx-1] (NaN -> 0), as cfloorf
  const float t = __fadd_rd(fminf(fmaxf(sxy.x, 0.0f), (float)(a.ncx - 1)), kMagic23);
  const int ic = magic_int(t);
  const float2 d = __fadd2_rn(sxy, make_float2(neg_magic_float(t), -(float)s));  // sx - ic, sy - s
  const float fx = clamp01f(d.x), fy = clamp01f(d.y);
  const float2 g = __fadd2_rn(make_float2(1.0f, 1.0f), make_float2(-fx, -fy));  // gx, gy
  const float2 wlo = __fmul2_rn(make_float2(g.x, fx), make_float2(g.y, g.y));    // w00, w10
  const float2 whi = __fmul2_rn(make_float2(g.x, fx), make_float2(fy, fy));      // w01, w11
  const float4 lo = tile[ic], hi = tile[a.ncx + ic];
  float2 e = __fmul2_rn(make_float2(wlo.x, wlo.x), make_float2(lo.x, lo.y));
  e = __ffma2_rn(make_float2(wlo.y, wlo.y), make_float2(lo.z, lo.w), e);
  e = __ffma2_rn(make_float2(whi.x, whi.x), make_float2(hi.x, hi.y), e);
  e = __ffma2_rn(make_float2(whi.y, whi.y), make_float2(hi.z, hi.w), e);
  Epx = e.x;
  Epy = e.y;
}

// fixed-point CIC weights: kFixBits = 18 fractional bits per axis and the
// cross term FX*FY rounded to a multiple of 2^(32-18), so the four weights
// are exact integers that sum to 2^32 per particle.  18 bits put the
// deposited charge within 4e-6 (relative) of the exact FP64 CIC weights on
// the same positions; 16 bits gave 1.5e-5.
constexpr int kFixBits = 18;
constexpr int kFixShift = 32 - kFixBits;  // node weight = offset << kFixShift
constexpr float kFixOne = (float)(1 << kFixBits);
struct CicFixed {
  int ic, jc;
  int FX, FY;  // offsets in the cell, kFixBits fractional bits, in [0, 2^kFixBits]
  int FXY;     // round(FX*FY / 2^kFixBits), in [0, 2^kFixBits]
  // the four node weights, formed where needed
  __device__ __forceinline__ long long w11() const { return (long long)FXY << kFixShift; }
  __device__ __forceinline__ long long w10() const { return ((long long)FX << kFixShift) - w11(); }
  __device__ __forceinline__ long long w01() const { return ((long long)FY << kFixShift) - w11(); }
  __device__ __forceinline__ long long w00() const {
    return 4294967296ll - (((long long)FX + FY) << kFixShift) + w11();
  }
};

// INSIDE: the caller knows 0 <= x < Lx and 0 <= y < Ly.  Then the cell
// indices and the offsets in the cell are >= 0, so of the clamps only the
// upper ones can act and the others are left out (same results).
template <bool INSIDE = false>
__device__ __forceinline__ CicFixed cic_fixed(const SimArgs &a, float x, float y) {
  CicFixed r;
  const float2 sxy = __fmul2_rn(make_float2(x, y), make_float2(a.inv_ds, a.inv_ds));
  if (INSIDE) {
    // sxy >= 0: floor of min(sxy, n-1) = min(floor(sxy), n-1), on the FP32 pipe
    const float2 t = __fadd2_rd(make_float2(fminf(sxy.x, (float)(a.ncx - 1)), fminf(sxy.y, (float)(a.ncy - 1))),
                                make_float2(kMagic23, kMagic23));
    r.ic = magic_int(t.x);
    r.jc = magic_int(t.y);
    const float2 d = __fadd2_rn(sxy, __ffma2_rd(t, make_float2(-1.0f, -1.0f), make_float2(kMagic23, kMagic23)));
    const float2 f = __fadd2_rn(__fmul2_rn(make_float2(fminf(d.x, 1.0f), fminf(d.y, 1.0f)),
                                           make_float2(kFixOne, kFixOne)),
                                make_float2(kMagic23, kMagic23));
    r.FX = magic_int(f.x);
    r.FY = magic_int(f.y);
  } else {
    r.ic = cfloorf(sxy.x, 0, a.ncx - 1);
    r.jc = cfloorf(sxy.y, 0, a.ncy - 1);
    const float2 d = __fadd2_rn(sxy, make_float2(-(float)r.ic, -(float)r.jc));
    const float2 f = __fmul2_rn(make_float2(clamp01f(d.x), clamp01f(d.y)), make_float2(kFixOne, kFixOne));
    r.FX = __float2int_rn(f.x);
    r.FY = __float2int_rn(f.y);
  }
  r.FXY = (int)(((unsigned long long)r.FX * (unsigned long long)r.FY +
                 (1ull << (kFixBits - 1))) >> kFixBits);
  return r;
}

// ---------------------------------------------------------------------------
// bulk-copy (TMA) + mbarrier helpers, inline PTX (sm_90+; used on sm_103a)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// make the initialised barriers visible to the bulk-copy (async) proxy
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// 1-D bulk copy global -> shared; completion is signalled on bar.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// bounded wait for phase `parity` of bar; false if it gave up
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = smem_addr(bar);
  for (int it = 0; it < (1 << 20); ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ bool finite4(const float4 &p) {
  return isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(p.w);
}

}  // namespace cupic
