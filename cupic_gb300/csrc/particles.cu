// particles.cu -- particle kernels of the GB300 PIC cycle.
//
// Storage: per species, y cell row j owns the segment
// parts[seg[j] .. seg[j]+cap[j]) of float4 {x,y,vx,vy}; its live particles
// are the prefix of length cnt[j].  One step's particle work is
//   k_push_deposit  gather + leapfrog + wrap + classify; stable in-place
//                   compaction of the row's stayers, staging of the movers
//                   to the neighbouring rows, and deposition of every moved
//                   particle into the next charge accumulator (fused; the
//                   reference runs fast_grid_to_particle, leap_frog_step,
//                   pDefragDown/Up, pRebracketing, bmHandler, pCyclicCC and
//                   fast_particle_to_grid as separate passes)
//   k_arrive        appends the movers from the rows below and above
//   k_inject        draws the injected flux of the step (cc.cu:179-256),
//                   appends it to the rows it falls in, deposits it
//   k_finalize      per-step counters, clock advance, charge buffer flip
#include <map>
#include <mutex>
#include <utility>

#include "cupic_internal.cuh"
#include "kernels.h"

namespace cupic {

namespace {

constexpr int kInjBlock = 1024;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ void raise_flags(Ctl *ctl, uint32_t f) {
  if (f) atomicOr(&ctl->step_flags, f);
}

// Charge deposition into shared memory by cell moments.  A particle with
// fixed-point offsets FX, FY in [0, 2^18] in its cell and cross term
// FXY = round(FX*FY / 2^18) (cic_fixed) gives its four nodes the weights
//   upper-right w11 = 2^14 FXY,          lower-right w10 = 2^14 FX - w11,
//   upper-left  w01 = 2^14 FY - w11,     lower-left  w00 = 2^32 - 2^14 (FX + FY) + w11,
// the CIC weights with FX*FY rounded to a multiple of 2^14; they sum to 2^32.
// Over the particles of a cell the four node sums follow from four integer
// moments M1 = count, MX = sum FX, MY = sum FY, MXY = sum FXY by the same
// formulas.  Shared memory atomics are native for 32-bit integers only, so
// a particle adds 1, FX, FY and FXY to the four unsigned moments of its
// cell, held in four arrays (one per moment): the lanes of a warp, on
// cells spread over the row, spread over the banks.  The moments of one
// species over at most kFoldParticles particles stay below 2^32; fold(q)
// turns them into int64 node sums times the species charge q, added to
// global memory, that often and at every change of species.  Deposits
// whose cell row is outside the tile go straight to global memory as int64
// node weights.
constexpr int kFoldParticles = (1 << (32 - kFixBits)) - 1;  // 16383 * 2^18 < 2^32

struct RhoMoments {
  unsigned *m;     // [4][ncr*ncx]: M1, MX, MY, MXY
  int crow0, ncr, ncx, nnx, nny;
  unsigned long long *g;

  __device__ __forceinline__ int cells() const { return ncr * ncx; }
  __device__ __forceinline__ void deposit(const SimArgs &a, float x, float y, int q) const {
    deposit(cic_fixed(a, x, y), q);
  }
  __device__ __forceinline__ void deposit(const CicFixed &c, int q) const {
    const int tr = c.jc - crow0;
    if (tr >= 0 && tr < ncr) {
      const int nc = cells();
      unsigned *mc = m + (tr * ncx + c.ic);
      atomicAdd(mc, 1u);
      atomicAdd(mc + nc, (unsigned)c.FX);
      atomicAdd(mc + 2 * nc, (unsigned)c.FY);
      atomicAdd(mc + 3 * nc, (unsigned)c.FXY);
    } else {
      const size_t n00 = (size_t)c.jc * nnx + c.ic;
      atomicAdd(&g[n00], (unsigned long long)(q * c.w00()));
      atomicAdd(&g[n00 + 1], (unsigned long long)(q * c.w10()));
      atomicAdd(&g[n00 + nnx], (unsigned long long)(q * c.w01()));
      atomicAdd(&g[n00 + nnx + 1], (unsigned long long)(q * c.w11()));
    }
  }
  // The common case without a branch: a particle inside the domain whose
  // cell row is within one of row s (this tile's middle row, crow0 = s-1)
  // adds its moments to the tile; returns its row step -1, 0 or 1, else 2
  // (and deposits nothing).  Out-of-domain or non-finite positions give
  // clamped in-range indices and no deposit.
  __device__ __forceinline__ int deposit_near(const SimArgs &a, const float4 &v, int s, bool live) const {
    const bool inside = v.y >= 0.0f && v.y < a.Ly && v.x >= 0.0f && v.x < a.Lx;
    const CicFixed c = cic_fixed<true>(a, v.x, v.y);
    const int dj = c.jc - s;
    const bool near = live && inside && dj >= -1 && dj <= 1;
    if (near) {
      const int nc = cells();
      unsigned *mc = m + ((dj + 1) * ncx + c.ic);
      atomicAdd(mc, 1u);
      atomicAdd(mc + nc, (unsigned)c.FX);
      atomicAdd(mc + 2 * nc, (unsigned)c.FY);
      atomicAdd(mc + 3 * nc, (unsigned)c.FXY);
    }
    return near ? dj : 2;
  }
  __device__ __forceinline__ void zero() const {
    for (int k = threadIdx.x; k < 4 * cells(); k += blockDim.x) m[k] = 0u;
  }
  __device__ __forceinline__ long long m1(int c) const { return (long long)m[c]; }
  __device__ __forceinline__ long long mx(int c) const { return (long long)m[cells() + c]; }
  __device__ __forceinline__ long long my(int c) const { return (long long)m[2 * cells() + c]; }
  __device__ __forceinline__ long long mxy(int c) const {
    return (long long)m[3 * cells() + c] << kFixShift;
  }
  // moments (of charge q particles) -> node sums added to global memory,
  // then clear the moments; callers __syncthreads() before, and before the
  // next deposit
  __device__ __forceinline__ void fold(int q) const {
    for (int k = threadIdx.x; k < (ncr + 1) * nnx; k += blockDim.x) {
      const int j = k / nnx, i = k - j * nnx;
      long long v = 0;
      if (i < ncx && j < ncr) {  // this node is the lower-left corner of cell (i, j)
        const int c = j * ncx + i;
        v += m1(c) * 4294967296ll - ((mx(c) + my(c)) << kFixShift) + mxy(c);
      }
      if (i >= 1 && j < ncr) {  // lower-right corner of cell (i-1, j)
        const int c = j * ncx + i - 1;
        v += (mx(c) << kFixShift) - mxy(c);
      }
      if (i < ncx && j >= 1) {  // upper-left corner of cell (i, j-1)
        const int c = (j - 1) * ncx + i;
        v += (my(c) << kFixShift) - mxy(c);
      }
      if (i >= 1 && j >= 1) {  // upper-right corner of cell (i-1, j-1)
        v += mxy((j - 1) * ncx + i - 1);
      }
      const int r = crow0 + j;
      if (v != 0 && r >= 0 && r < nny)
        atomicAdd(&g[(size_t)r * nnx + i], (unsigned long long)(q * v));
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 4 * cells(); k += blockDim.x) m[k] = 0u;
  }
};

__host__ __device__ constexpr size_t rho_moment_bytes(int ncr, int ncx) {
  return (size_t)4 * ncr * ncx * sizeof(unsigned);
}

// classification of a pushed particle listed in row s (s < 0: injected)
struct Cls {
  int dest;  // row, kRowAbsorbed or kRowRemoved
  uint32_t flag;
};

__device__ __forceinline__ Cls classify(const SimArgs &a, const float4 &p, int s) {
  if (!finite4(p)) return {kRowRemoved, CUPIC_FLAG_NONFINITE};
  if (p.y < 0.0f) return {kRowAbsorbed, 0u};
  if (p.y >= a.Ly) return {kRowRemoved, 0u};
  uint32_t f = 0;
  if (p.x < 0.0f || p.x >= a.Lx) f |= CUPIC_FLAG_XRANGE;
  const int d = row_of(a, p.y);
  if (s >= 0 && (d > s + 1 || d < s - 1)) return {s, f | CUPIC_FLAG_CFL};
  return {d, f};
}

// A pushed particle of row s, settled in two parts: RhoMoments::deposit_near()
// takes the common case without a branch (inside the domain, a row step of
// at most one), and settle_far() the rest: a row step beyond one (deposited
// to global memory, CFL flag) or a position outside the domain (classify()).
// Both return 0 stay, 1 up, 2 down, 3 absorbed or removed.  x = wrap(x0 +
// dt vx) and y = y0 + dt vy are finite only if vx and vy are (dt = 0 turns
// an infinite velocity into NaN), so a particle with both coordinates
// inside the domain is finite4 and needs no further test but the row step;
// its row is the deposit's cell row.
__device__ __forceinline__ int settle_far(const SimArgs &a, const float4 &v, int s, const RhoMoments &T,
                                          int q, uint32_t &fl, unsigned &nabs, unsigned &nrem) {
  if (v.y >= 0.0f && v.y < a.Ly && v.x >= 0.0f && v.x < a.Lx) {
    T.deposit(cic_fixed<true>(a, v.x, v.y), q);
    fl |= CUPIC_FLAG_CFL;
    return 0;
  }
  const Cls c = classify(a, v, s);
  fl |= c.flag;
  if (c.dest == kRowAbsorbed) {
    ++nabs;
    return 3;
  }
  if (c.dest == kRowRemoved) {
    ++nrem;
    return 3;
  }
  T.deposit(a, v.x, v.y, q);
  return c.dest == s ? 0 : (c.dest == s + 1 ? 1 : 2);
}

// The same in one call, with a branch: the push kernels of 2 particles a
// thread (the batched ones, held to 64 registers) run faster this way.
__device__ __forceinline__ int settle(const SimArgs &a, const float4 &v, int s, const RhoMoments &T,
                                      int q, uint32_t &fl, unsigned &nabs, unsigned &nrem) {
  if (v.y >= 0.0f && v.y < a.Ly && v.x >= 0.0f && v.x < a.Lx) {
    const CicFixed c = cic_fixed<true>(a, v.x, v.y);
    T.deposit(c, q);
    const int dj = c.jc - s;  // c.jc == row_of(a, v.y)
    if (dj == 0) return 0;
    if (dj == 1) return 1;
    if (dj == -1) return 2;
    fl |= CUPIC_FLAG_CFL;
    return 0;
  }
  return settle_far(a, v, s, T, q, fl, nabs, nrem);
}

}  // namespace

// ---------------------------------------------------------------------------
// initial plasma (init.cu:159-179, with the project's counter-based draws)
// ---------------------------------------------------------------------------
__global__ void k_init_particles(SimArgs a) {
  const int j = blockIdx.x, sp = blockIdx.y;
  const SpeciesDev &S = a.sp[sp];
  float4 *row = S.parts + S.seg[j];
  const double sig = a.sig[sp];
  for (int k = threadIdx.x; k < a.ppr; k += blockDim.x) {
    const uint4 r = philox4x32_10(
        make_uint4((uint32_t)k, (uint32_t)j, 0u, (uint32_t)((kPurposeInit << 8) | sp)), a.k0, a.k1);
    const double x = u01(r.x) * a.Lx_d;
    const double y = ((double)j + u01(r.y)) * a.ds_d;
    const double rr = sqrt(-2.0 * dev_log(u01(r.z)));
    double sn, cs;
    dev_sincos2pi(u01(r.w), &sn, &cs);
    float4 p = make_float4((float)x, (float)y, (float)(sig * (rr * cs)), (float)(sig * (rr * sn)));
    p.x = wrap_x(a, p.x);
    for (int it = 0; it < 16 && row_of(a, p.y) > j; ++it) p.y = nextafterf(p.y, 0.0f);
    for (int it = 0; it < 16 && row_of(a, p.y) < j; ++it) p.y = nextafterf(p.y, a.Ly);
    row[k] = p;
  }
  if (threadIdx.x == 0) S.cnt[j] = a.ppr;
}

// ---------------------------------------------------------------------------
// charge deposition of the current particles into rho[ctl->cur]
// (mesh.cu:162-293; int64 fixed point, so the sum is order independent)
// ---------------------------------------------------------------------------
__global__ void k_deposit(SimArgs a) {
  extern __shared__ unsigned dtile[];
  const int s = blockIdx.x, nnx = a.nnx, ncx = a.ncx;
  RhoMoments T{dtile, s, 1, ncx, nnx, a.nny, a.rho[a.ctl->cur]};
  T.zero();
  __syncthreads();
  for (int sp = 0; sp < 2; ++sp) {
    const SpeciesDev &S = a.sp[sp];
    const float4 *row = S.parts + S.seg[s];
    const int n = S.cnt[s];
    const int q = sp == 0 ? -1 : 1;
    int since = 0;
    for (int base = 0; base < n; base += blockDim.x) {
      const int k = base + threadIdx.x;
      if (k < n) {
        const float4 p = row[k];
        T.deposit(a, p.x, p.y, q);
      }
      since += blockDim.x;
      if (since + (int)blockDim.x > kFoldParticles) {  // block-uniform
        __syncthreads();
        T.fold(q);
        __syncthreads();
        since = 0;
      }
    }
    __syncthreads();
    T.fold(q);  // a species' moments are folded before the next one's
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// set-up kernels, so that a context's set-up is ordered on its own stream
// and never waits on the host for the device
// ---------------------------------------------------------------------------
// uniform row layout: segment j at j*capj, capacity capj, no particles
__global__ void k_uniform_layout(SpeciesDev S, int ncy, int capj) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < ncy; j += gridDim.x * blockDim.x) {
    S.seg[j] = (int64_t)j * capj;
    S.cap[j] = capj;
    S.cnt[j] = S.nstay[j] = S.nup[j] = S.ndown[j] = 0;
  }
}

// the clocks of the control block (the first fields of Ctl)
__global__ void k_set_time(Ctl *ctl, int64_t step, double t, double tin_e, double tin_i) {
  ctl->step = step;
  ctl->t = t;
  ctl->tin[0] = tin_e;
  ctl->tin[1] = tin_i;
  ctl->tin_set[0] = tin_e >= 0 ? 1 : 0;
  ctl->tin_set[1] = tin_i >= 0 ? 1 : 0;
}

// phi = (1 - j/ncy) phi_p on node row j (init.cu:235-241), in FP64, the
// FP32 copy rounded from it
__global__ void k_linear_phi(SimArgs a, double phi_p, double *phi64) {
  const int j = blockIdx.y;
  const double v = __dmul_rn(__dsub_rn(1.0, __ddiv_rn((double)j, (double)a.ncy)), phi_p);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nnx; i += gridDim.x * blockDim.x) {
    a.phi[(size_t)j * a.nnx + i] = (float)v;
    if (phi64) phi64[(size_t)j * a.nnx + i] = v;
  }
}

// zero the accumulator the next deposit writes (rho[cur^1])
__global__ void k_zero_next_rho(SimArgs a) {
  if (halted(a.ctl)) return;
  unsigned long long *r = a.rho[a.ctl->cur ^ 1];
  const size_t n = (size_t)a.nnx * a.nny;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    r[k] = 0ull;
}

// ---------------------------------------------------------------------------
// leapfrog start: v -= dt/2 q E / m (init.cu:264-323, 793-833)
// ---------------------------------------------------------------------------
__global__ void k_leapfrog_start(SimArgs a) {
  extern __shared__ float2 etile[];
  const int s = blockIdx.x;
  for (int k = threadIdx.x; k < 2 * a.nnx; k += blockDim.x) etile[k] = a.E[(size_t)s * a.nnx + k];
  __syncthreads();
  for (int sp = 0; sp < 2; ++sp) {
    const SpeciesDev &S = a.sp[sp];
    float4 *row = S.parts + S.seg[s];
    const int n = S.cnt[s];
    const float h = a.mhdtqm[sp];
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      float4 p = row[k];
      float ex, ey;
      gather_tile(a, etile, p.x, p.y, s, ex, ey);
      p.z = __fmaf_rn(h, ex, p.z);
      p.w = __fmaf_rn(h, ey, p.w);
      row[k] = p;
    }
  }
}

// ---------------------------------------------------------------------------
// fused push + wrap + row binning + deposition, one block per (cell row s,
// species) unit (particles.cu:110-231, cc.cu:303-810, mesh.cu:162-293)
//
// The row's particles stream through a ring of kStages shared-memory chunks
// of CH = PB*PPT particles filled by 1-D bulk copies (TMA) that run
// kStages-1 chunks ahead of the compute.  Thread t handles particles
// j*PB + t (j < PPT) of a chunk; one block-wide scan per chunk gives every
// stayer its slot (the stayers are compacted in place, keeping their order)
// and every mover its slot in the staging buffer of its new row.  In-place
// compaction is safe because no write goes past the chunk being processed
// and every later chunk is disjoint from it.
// ---------------------------------------------------------------------------
namespace {
constexpr int kPB = 256;       // threads of the single-context push (3 blocks per SM)
// particles per thread per chunk: 4 for the single-context push's 256-thread
// blocks (1024-particle chunks: half the block barriers per particle of
// 2, and four independent particles per thread; 3.5% faster at 512x2048
// although the 65 KB of shared memory leave 3 blocks per SM instead of 4),
// 2 for the batched ones
template <int PB>
constexpr int ppt() { return PB == 256 ? 4 : 2; }
constexpr int kStages = 2;     // chunks in flight
// a chunk's scan has one entry per (particle slot j, warp), 32 particles each

// three counts packed in 32 bits: 10 + 11 + 11 bits, enough for every
// exclusive prefix of a chunk (at most 32*(32-1) = 992)
__device__ __forceinline__ uint32_t pack3(int a, int b, int c) {
  return (uint32_t)a | ((uint32_t)b << 10) | ((uint32_t)c << 21);
}
__device__ __forceinline__ uint32_t field0(uint32_t v) { return v & 0x3ffu; }
__device__ __forceinline__ uint32_t field1(uint32_t v) { return (v >> 10) & 0x7ffu; }
__device__ __forceinline__ uint32_t field2(uint32_t v) { return v >> 21; }
}  // namespace

size_t push_smem_bytes(int nnx, int pb) {
  return (size_t)kStages * pb * (pb == 256 ? 4 : 2) * sizeof(float4) + rho_moment_bytes(3, nnx - 1) +
         (size_t)2 * (nnx - 1) * sizeof(float4);
}

// NEAR: the four particles of a thread settle their common case without a
// branch (RhoMoments::deposit_near), the rest after (settle_far).  Their
// chains then interleave, at 72 registers a thread instead of 64.
template <int PB, bool NEAR = false>
__device__ __forceinline__ void push_unit(const SimArgs &a, const int s, const int sp,
                                          unsigned char *push_raw) {
  constexpr int NW = PB / 32;
  constexpr int kPPT = ppt<PB>();
  constexpr int CH = PB * kPPT;  // particles per chunk
  constexpr int NE = kPPT * NW;  // scan entries per chunk, (j, warp) in j-major order
  static_assert(NE <= 32, "one warp scans a chunk's entries");
  constexpr int kCheckChunks = 8192 / CH;  // chunks between fold checks
  static_assert((kCheckChunks + 1) * CH < kFoldParticles, "a fold check interval fits the moments");
  if (halted(a.ctl)) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nnx = a.nnx;
  const int ncx = a.ncx;
  float4 *stage = reinterpret_cast<float4 *>(push_raw);
  // node rows s, s+1 as node pairs (gather_pairs): 2 x ncx entries
  float4 *etile = stage + kStages * CH;
  unsigned *tmom = reinterpret_cast<unsigned *>(etile + 2 * ncx);  // cell rows s-1..s+1
  __shared__ __align__(8) uint64_t full[kStages];
  __shared__ uint2 wmask[2][NE];  // per-entry category ballots, alternate chunks
  __shared__ unsigned long long s_cnt[2];
  __shared__ unsigned s_cmax[NW];  // per-warp largest cell count, at a fold check

  Ctl *ctl = a.ctl;
  const SpeciesDev &S = a.sp[sp];
  const int nn = S.cnt[s];
  const int nch = (nn + CH - 1) / CH;
  float4 *row = S.parts + S.seg[s];

  if (tid == 0) {
    for (int i = 0; i < kStages; ++i) mbar_init(&full[i], 1);
    fence_mbar_init();
    s_cnt[0] = s_cnt[1] = 0ull;
  }
  __syncthreads();
  if (tid == 0) {
    for (int k = 0; k < kStages && k < nch; ++k) {
      const int cnt = min(CH, nn - k * CH);
      mbar_arrive_expect_tx(&full[k], (uint32_t)cnt * 16u);
      bulk_g2s(stage + k * CH, row + (size_t)k * CH, (uint32_t)cnt * 16u, &full[k]);
    }
  }
  RhoMoments T{tmom, s - 1, 3, ncx, nnx, a.nny, a.rho[ctl->cur ^ 1]};
  T.zero();
  for (int k = tid; k < 2 * ncx; k += PB) {
    const int r = k >= ncx ? 1 : 0, i = k - r * ncx;
    const float2 *er = a.E + (size_t)(s + r) * nnx + i;
    const float2 e0 = er[0], e1 = er[1];
    etile[k] = make_float4(e0.x, e0.y, e1.x, e1.y);
  }
  __syncthreads();

  uint32_t fl = 0;
  unsigned nabs = 0u, nrem = 0u;
  const uint32_t lt = (1u << lane) - 1u;
  const float dtqm = a.dtqm[sp];
  const int qc = sp == 0 ? -1 : 1;
  float4 *sup = S.stage_up + (size_t)s * S.stage_cap;
  float4 *sdn = S.stage_down + (size_t)s * S.stage_cap;
  int c_stay = 0, c_up = 0, c_dn = 0;
  for (int k = 0; k < nch; ++k) {
    const int st = k % kStages;
    if (!mbar_wait(&full[st], (uint32_t)((k / kStages) & 1))) fl |= CUPIC_FLAG_TIMEOUT;
    const int cnt = min(CH, nn - k * CH);
    float4 p[kPPT];
    int cat[kPPT];  // 0 stay, 1 up, 2 down, 3 none
    if constexpr (NEAR) {
      static_assert(kPPT == 4, "the branch-free form is written for four particles a thread");
      bool rare = false;
#pragma unroll
      for (int j = 0; j < kPPT; ++j) {
        const int idx = j * PB + tid;
        const bool live = idx < cnt;
        // a slot past the chunk's end computes on stale stage words: every
        // index it forms is clamped in range, and it deposits and stores nothing
        float4 v = stage[st * CH + idx];
        float ex, ey;
        gather_pairs(a, etile, v.x, v.y, s, ex, ey);
        // v += dtqm E, then r += dt v, both components per packed operation
        const float2 vel = __ffma2_rn(make_float2(dtqm, dtqm), make_float2(ex, ey), make_float2(v.z, v.w));
        const float2 pos = __ffma2_rn(make_float2(a.dt, a.dt), vel, make_float2(v.x, v.y));
        v = make_float4(wrap_x(a, pos.x), pos.y, vel.x, vel.y);
        const int dj = T.deposit_near(a, v, s, live);
        cat[j] = dj == 0 ? 0 : (dj == 1 ? 1 : (dj == -1 ? 2 : 3));
        rare |= live && cat[j] == 3;
        p[j] = v;
      }
      if (rare) {
#pragma unroll
        for (int j = 0; j < kPPT; ++j)
          if (j * PB + tid < cnt && cat[j] == 3) cat[j] = settle_far(a, p[j], s, T, qc, fl, nabs, nrem);
      }
    } else {
#pragma unroll
      for (int j = 0; j < kPPT; ++j) {
        const int idx = j * PB + tid;
        cat[j] = 3;
        if (idx < cnt) {
          float4 v = stage[st * CH + idx];
          float ex, ey;
          gather_pairs(a, etile, v.x, v.y, s, ex, ey);
          const float2 vel = __ffma2_rn(make_float2(dtqm, dtqm), make_float2(ex, ey), make_float2(v.z, v.w));
          const float2 pos = __ffma2_rn(make_float2(a.dt, a.dt), vel, make_float2(v.x, v.y));
          v = make_float4(wrap_x(a, pos.x), pos.y, vel.x, vel.y);
          cat[j] = settle(a, v, s, T, qc, fl, nabs, nrem);
          p[j] = v;
        }
      }
    }
    // category bits of the warp's lanes: 00 stay, 01 up, 10 down, 11 none
    uint32_t b0[kPPT], b1[kPPT];
    uint2 *wm = wmask[k & 1];
#pragma unroll
    for (int j = 0; j < kPPT; ++j) {
      b0[j] = __ballot_sync(kFull, cat[j] & 1);
      b1[j] = __ballot_sync(kFull, cat[j] & 2);
      if (lane == 0) wm[j * NW + warp] = make_uint2(b0[j], b1[j]);
    }
    // fold check, every kCheckChunks chunks (block-uniform): the largest
    // cell count so far, read while this chunk's deposits may still land
    const bool check = (k % kCheckChunks) == kCheckChunks - 1 && k + 1 < nch;
    if (check) {
      unsigned c = 0u;
      for (int i = tid; i < T.cells(); i += PB) c = max(c, T.m[i]);
      c = __reduce_max_sync(kFull, c);
      if (lane == 0) s_cmax[warp] = c;
    }
    __syncthreads();  // the only block barrier of a chunk
    // every thread holds its particles: refill this stage with chunk k+kStages
    if (tid == 0 && k + kStages < nch) {
      const int k2 = k + kStages;
      const int cnt2 = min(CH, nn - k2 * CH);
      mbar_arrive_expect_tx(&full[st], (uint32_t)cnt2 * 16u);
      bulk_g2s(stage + st * CH, row + (size_t)k2 * CH, (uint32_t)cnt2 * 16u, &full[st]);
    }
    // Every warp sums the chunk's NE entries itself (no second barrier): the
    // exclusive prefix of entry e is the sum of entries 0..e-1.  Exclusive
    // prefixes are at most 32*(NE-1) < 1024 per field, so the packed sums
    // never carry between fields; the chunk totals come from the last entry
    // field by field.
    uint32_t v = 0u;  // lane e: the packed counts of entry e
    if (lane < NE) {
      const uint2 m = wm[lane];
      v = pack3(__popc(~(m.x | m.y)), __popc(m.x & ~m.y), __popc(m.y & ~m.x));
    }
    const uint32_t exl = __reduce_add_sync(kFull, lane < NE - 1 ? v : 0u);
    const uint32_t vl = __shfl_sync(kFull, v, NE - 1);
#pragma unroll
    for (int j = 0; j < kPPT; ++j) {
      const uint32_t off = __reduce_add_sync(kFull, lane < j * NW + warp ? v : 0u);
      const int c = cat[j];
      if (c < 3) {
        // one store: the slot among the lanes of the same category
        const uint32_t m0 = (c & 1) ? kFull : 0u, m1 = (c & 2) ? kFull : 0u;
        const uint32_t same = ~((b0[j] ^ m0) | (b1[j] ^ m1));
        const int sh = c == 0 ? 0 : (c == 1 ? 10 : 21);
        const int base = c == 0 ? c_stay : (c == 1 ? c_up : c_dn);
        const int pos = base + (int)((off >> sh) & (c == 0 ? 0x3ffu : 0x7ffu)) + __popc(same & lt);
        float4 *dst = c == 0 ? row : (c == 1 ? sup : sdn);
        if (c == 0 || pos < S.stage_cap) dst[pos] = p[j]; else fl |= CUPIC_FLAG_STAGE;
      }
    }
    c_stay += (int)(field0(exl) + field0(vl));
    c_up += (int)(field1(exl) + field1(vl));
    c_dn += (int)(field2(exl) + field2(vl));
    // Fold before the moments could overflow.  A cell's moments stay below
    // 2^32 while its count stays at most kFoldParticles.  The count read at
    // the check misses at most this chunk's CH deposits, and the next check
    // comes kCheckChunks chunks later, so without a fold no cell can pass
    // cmax + (kCheckChunks + 1) * CH before then.  At ordinary densities
    // that stays far below the limit and a row folds only at its end.  The
    // barrier after a fold orders the clearing before the next deposits.
    if (check) {
      unsigned cmax = 0u;
#pragma unroll
      for (int w = 0; w < NW; ++w) cmax = max(cmax, s_cmax[w]);
      if (cmax + (unsigned)((kCheckChunks + 1) * CH) > (unsigned)kFoldParticles) {
        __syncthreads();
        T.fold(qc);
        __syncthreads();
      }
    }
  }
  if (tid == 0) {
    S.nstay[s] = c_stay;
    S.nup[s] = min(c_up, S.stage_cap);
    S.ndown[s] = min(c_dn, S.stage_cap);
  }
  const unsigned wa = __reduce_add_sync(kFull, nabs);
  const unsigned wr = __reduce_add_sync(kFull, nrem);
  if (lane == 0 && (wa | wr)) {
    atomicAdd(&s_cnt[0], (unsigned long long)wa);
    atomicAdd(&s_cnt[1], (unsigned long long)wr);
  }
  __syncthreads();
  if (tid == 0) {
    if (s_cnt[0]) atomicAdd(&ctl->absorbed[sp], s_cnt[0]);
    if (s_cnt[1]) atomicAdd(&ctl->removed[sp], s_cnt[1]);
  }
  T.fold(qc);
  fl = __reduce_or_sync(kFull, fl);
  if (lane == 0) raise_flags(ctl, fl);
}

// block 2s + sp pushes species sp of row s: both species of a row are
// independent units of equal size, which halves the tail of the last wave.
// Rows whose tiles leave room for 4 blocks per SM (up to about 300 cells)
// take k_push_deposit_narrow, the branching settle at 64 registers, so
// that 4 blocks fit; wider rows, held to 3 blocks by shared memory anyway,
// take the branch-free settle at 72 registers (1.7% faster at 512 cells,
// and 5% slower on the batched step's meshes of 128 and 256 cells, where it
// costs the fourth block).  The narrow kernel keeps the bound of 3 blocks:
// bounding it to 4 made the compiler take 61 registers and the batched
// step 2.6% slower.
__global__ void __launch_bounds__(kPB, 3) k_push_deposit(SimArgs a) {
  extern __shared__ __align__(128) unsigned char push_raw[];
  push_unit<kPB, true>(a, blockIdx.x >> 1, blockIdx.x & 1, push_raw);
}
__global__ void __launch_bounds__(kPB, 3) k_push_deposit_narrow(SimArgs a) {
  extern __shared__ __align__(128) unsigned char push_raw[];
  push_unit<kPB, false>(a, blockIdx.x >> 1, blockIdx.x & 1, push_raw);
}

// many contexts in one launch: block 2b + sp pushes species sp of work[b] =
// {instance, row}; PB = 128 for short rows (eight blocks per SM: a short
// row's unit is mostly set-up, which more resident blocks overlap), 512
// otherwise
template <int PB>
__global__ void __launch_bounds__(PB, PB == 128 ? 8 : 2)
    k_push_deposit_batch(const SimArgs *__restrict__ inst, const int2 *__restrict__ work) {
  extern __shared__ __align__(128) unsigned char push_raw[];
  // the instance's arguments in shared memory: read there as needed instead
  // of held in registers
  __shared__ __align__(16) SimArgs sa;
  const int2 w = work[blockIdx.x >> 1];
  static_assert(sizeof(SimArgs) % 4 == 0, "");
  const unsigned *src = reinterpret_cast<const unsigned *>(inst + w.x);
  unsigned *dst = reinterpret_cast<unsigned *>(&sa);
  for (int k = threadIdx.x; k < (int)(sizeof(SimArgs) / 4); k += PB) dst[k] = src[k];
  __syncthreads();
  push_unit<PB>(sa, w.y, blockIdx.x & 1, push_raw);
}

// ---------------------------------------------------------------------------
// append the movers: row d = [stayed] + [up from d-1] + [down from d+1]
// ---------------------------------------------------------------------------
__device__ __forceinline__ void arrive_row(const SimArgs &a, const int d, const int sp) {
  if (halted(a.ctl)) return;
  const SpeciesDev &S = a.sp[sp];
  const int ns = S.nstay[d];
  const int nb = d > 0 ? S.nup[d - 1] : 0;
  const int na = d + 1 < a.ncy ? S.ndown[d + 1] : 0;
  const int capd = S.cap[d];
  float4 *row = S.parts + S.seg[d];
  if (nb) {
    const float4 *src = S.stage_up + (size_t)(d - 1) * S.stage_cap;
    for (int k = threadIdx.x; k < nb; k += blockDim.x)
      if (ns + k < capd) row[ns + k] = src[k];
  }
  if (na) {
    const float4 *src = S.stage_down + (size_t)(d + 1) * S.stage_cap;
    for (int k = threadIdx.x; k < na; k += blockDim.x)
      if (ns + nb + k < capd) row[ns + nb + k] = src[k];
  }
  if (threadIdx.x == 0) {
    const int tot = ns + nb + na;
    if (tot > capd) raise_flags(a.ctl, CUPIC_FLAG_CAPACITY);
    S.cnt[d] = min(tot, capd);
  }
}

__global__ void k_arrive(SimArgs a) { arrive_row(a, blockIdx.x, blockIdx.y); }

// many contexts: one warp per (row, species) task t = 2 * work index +
// species, eight per block -- most rows of a batch move few particles, so a
// block per row would be mostly set-up
constexpr int kArriveWarps = 8;
__global__ void __launch_bounds__(32 * kArriveWarps)
    k_arrive_batch(const SimArgs *__restrict__ inst, const int2 *__restrict__ work, int ntask) {
  const int t = blockIdx.x * kArriveWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (t >= ntask) return;
  const int2 w = work[t >> 1];
  const SimArgs &a = inst[w.x];
  if (halted(a.ctl)) return;
  const int d = w.y, sp = t & 1;
  const SpeciesDev &S = a.sp[sp];
  const int ns = S.nstay[d];
  const int nb = d > 0 ? S.nup[d - 1] : 0;
  const int na = d + 1 < a.ncy ? S.ndown[d + 1] : 0;
  const int capd = S.cap[d];
  float4 *row = S.parts + S.seg[d];
  if (nb) {
    const float4 *up = S.stage_up + (size_t)(d - 1) * S.stage_cap;
    for (int k = lane; k < nb; k += 32)
      if (ns + k < capd) row[ns + k] = up[k];
  }
  if (na) {
    const float4 *dn = S.stage_down + (size_t)(d + 1) * S.stage_cap;
    for (int k = lane; k < na; k += 32)
      if (ns + nb + k < capd) row[ns + nb + k] = dn[k];
  }
  if (lane == 0) {
    const int tot = ns + nb + na;
    if (tot > capd) raise_flags(a.ctl, CUPIC_FLAG_CAPACITY);
    S.cnt[d] = min(tot, capd);
  }
}

// ---------------------------------------------------------------------------
// room check, between the push and the arrivals.  The reference reallocates
// its particle array at every boundary call (cc.cu:195,260), so it never
// runs out of room; here rows have fixed capacities.  Row d must take its
// stayers, the movers staged for it from rows d-1 and d+1 and the particles
// injected into it.  When one row of a species cannot, the run halts before
// any particle is written: the later kernels of the step and of the steps
// after it return at once, and the host grows the rows that are short,
// completes the step and runs the steps that were skipped.  Nothing waits for
// the host on the way, and the results are those of a run with larger rows.
// The check writes nothing but the flag, so it runs in a halted run too
// (it then finds the same rows short again) and needs no gate.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void room_check(const SimArgs &a, const int sp, int *inj) {
  Ctl *ctl = a.ctl;
  const SpeciesDev &S = a.sp[sp];
  const int ncy = a.ncy;
  for (int k = threadIdx.x; k < ncy; k += blockDim.x) inj[k] = 0;
  __syncthreads();
  const int ne = ctl->inj_gen[sp];
  for (int k = threadIdx.x; k < ne; k += blockDim.x) {
    const int d = S.inj_d[k];
    if (d >= 0 && d < ncy) atomicAdd(&inj[d], 1);
  }
  __syncthreads();
  int over = 0;
  for (int d = threadIdx.x; d < ncy; d += blockDim.x) {
    const long long need = (long long)S.nstay[d] + (d > 0 ? S.nup[d - 1] : 0) +
                           (d + 1 < ncy ? S.ndown[d + 1] : 0) + inj[d];
    over |= need > (long long)S.cap[d];
  }
  if (__syncthreads_or(over) && threadIdx.x == 0) atomicExch(&ctl->halt, 1);
}

constexpr int kRoomBlock = 512;

__global__ void __launch_bounds__(kRoomBlock) k_room(SimArgs a) {
  extern __shared__ int inj_rows[];
  room_check(a, blockIdx.x, inj_rows);
}

// grid (species, instance)
__global__ void __launch_bounds__(kRoomBlock) k_room_batch(const SimArgs *__restrict__ inst) {
  extern __shared__ int inj_rows[];
  room_check(inst[blockIdx.y], blockIdx.x, inj_rows);
}

// a species moved to a larger layout: the first keep[j] particles of row j
// from old + oseg[j] to parts + nseg[j], in order (one block per row)
__global__ void k_move_rows(const float4 *__restrict__ old, const int64_t *__restrict__ oseg,
                            float4 *__restrict__ parts, const int64_t *__restrict__ nseg,
                            const int32_t *__restrict__ keep) {
  const int j = blockIdx.x;
  const int n = keep[j];
  const float4 *src = old + oseg[j];
  float4 *dst = parts + nseg[j];
  for (int k = threadIdx.x; k < n; k += blockDim.x) dst[k] = src[k];
}

// ---------------------------------------------------------------------------
// injection of the half-Maxwellian flux at y = Ly (cc.cu:179-256), in three
// kernels:
//   k_inject_sched   the step's count and the injection time of every draw,
//                    accumulated one dtin at a time as the reference does
//   k_inject_gen     one thread per draw: Philox4x32-10 draw {k, i_lo, i_hi,
//                    1<<8|sp}, Maxwellian/Rayleigh velocities, field at the
//                    injection point, the partial-step push, classification
//   k_inject_append  one block per species: stable rank of each draw within
//                    its destination row, append, deposit
// ---------------------------------------------------------------------------
__device__ __forceinline__ void inject_sched(const SimArgs &a, const int sp) {
  const SpeciesDev &S = a.sp[sp];
  Ctl *ctl = a.ctl;
  if (halted(ctl)) return;
  const double t = ctl->t;
  const double fpt = t + a.dt_d;
  if (!ctl->tin_set[sp]) {
    ctl->tin[sp] = t + a.dtin[sp];
    ctl->tin_set[sp] = 1;
  }
  double tin = ctl->tin[sp];
  int in = 0;
  if (tin < fpt) in = 1 + (int)((fpt - tin) / a.dtin[sp]);
  const int ne = in < S.inj_cap ? in : S.inj_cap;
  if (in > ne) atomicOr(&ctl->step_flags, (uint32_t)CUPIC_FLAG_CAPACITY);
  for (int k = 0; k < in; ++k) {
    if (k < ne) S.inj_tin[k] = tin;
    tin += a.dtin[sp];
  }
  ctl->tin[sp] = tin;
  ctl->inj_count[sp] = in;
  ctl->inj_gen[sp] = ne;
}

__global__ void k_inject_sched(SimArgs a) {
  if (threadIdx.x < 2) inject_sched(a, threadIdx.x);
}

// thread 2*i + sp handles species sp of instance i
__global__ void k_inject_sched_batch(const SimArgs *__restrict__ inst, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 2 * n) inject_sched(inst[t >> 1], t & 1);
}

__device__ __forceinline__ void inject_gen(const SimArgs &a, const int sp, const int k) {
  const Ctl *ctl = a.ctl;
  if (halted(ctl)) return;
  const int ne = ctl->inj_gen[sp];
  if (k >= ne) return;
  const SpeciesDev &S = a.sp[sp];
  const double t = ctl->t, fpt = t + a.dt_d, fvt = t + 0.5 * a.dt_d;
  const double sig = a.sig[sp], qm = a.qm[sp];
  const int64_t step = ctl->step;
  const size_t top = (size_t)(a.nny - 1) * a.nnx;
  const uint4 r = philox4x32_10(make_uint4((uint32_t)k, (uint32_t)step, (uint32_t)((uint64_t)step >> 32),
                                           (uint32_t)((kPurposeInject << 8) | sp)),
                                a.k0, a.k1);
  double x = u01(r.x) * a.Lx_d;
  double sn, cs;
  dev_sincos2pi(u01(r.z), &sn, &cs);
  double vx = sig * (sqrt(-2.0 * dev_log(u01(r.y))) * cs);
  double vy = -(sig * sqrt(-2.0 * dev_log(u01(r.w))));
  const int ic = cfloord(x * a.inv_ds_d, 0, a.ncx - 1);
  const double fx = clamp01d(x * a.inv_ds_d - (double)ic);
  const float2 e0 = a.E[top + ic], e1 = a.E[top + ic + 1];
  const double epx = (1.0 - fx) * (double)e0.x + fx * (double)e1.x;
  const double epy = (1.0 - fx) * (double)e0.y + fx * (double)e1.y;
  const double tin = S.inj_tin[k];
  const double dp = fpt - tin, dv = fvt - tin;
  x = x + dp * vx;
  const double y = a.Ly_d + dp * vy;
  vx = vx + dv * (qm * epx);
  vy = vy + dv * (qm * epy);
  float4 p = make_float4((float)x, (float)y, (float)vx, (float)vy);
  p.x = wrap_x(a, p.x);
  const Cls c = classify(a, p, -1);
  if (c.flag) atomicOr(&a.ctl->step_flags, c.flag);
  S.inj_p[k] = p;
  S.inj_d[k] = c.dest;
}

__global__ void k_inject_gen(SimArgs a) {
  inject_gen(a, blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x);
}

// grid (draw blocks, species, instance)
__global__ void k_inject_gen_batch(const SimArgs *__restrict__ inst) {
  inject_gen(inst[blockIdx.z], blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x);
}

__device__ __forceinline__ void inject_append(const SimArgs &a, const int sp, int *running) {
  // running: [ncy] injected per destination row
  constexpr int NW = kInjBlock / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const SpeciesDev &S = a.sp[sp];
  Ctl *ctl = a.ctl;
  if (halted(ctl)) return;
  __shared__ unsigned s_rem;
  if (tid == 0) s_rem = 0;
  for (int k = tid; k < a.ncy; k += kInjBlock) running[k] = 0;
  __syncthreads();
  const int ne = ctl->inj_gen[sp];
  const long long q = sp == 0 ? -1 : 1;
  unsigned long long *rho_next = a.rho[ctl->cur ^ 1];
  uint32_t fl = 0;
  unsigned nrem = 0;
  for (int base = 0; base < ne; base += kInjBlock) {
    const int k = base + tid;
    int d = kRowRemoved;
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
    if (k < ne) {
      p = S.inj_p[k];
      d = S.inj_d[k];
      if (d < 0) ++nrem;
    }
    // stable rank of each draw within its destination row, in draw order
    const int key = d >= 0 ? d : -1 - lane;
    const uint32_t grp = __match_any_sync(kFull, key);
    const int leader = __ffs(grp) - 1;
    const int rank = __popc(grp & ((1u << lane) - 1u));
    int basev = 0;
    for (int w = 0; w < NW; ++w) {
      if (warp == w && d >= 0 && lane == leader) {
        basev = running[d];
        running[d] = basev + __popc(grp);
      }
      __syncthreads();
    }
    const int b0 = __shfl_sync(kFull, basev, leader);
    if (d >= 0) {
      const int pos = S.cnt[d] + b0 + rank;
      if (pos < S.cap[d]) {
        S.parts[S.seg[d] + pos] = p;
        const CicFixed c = cic_fixed(a, p.x, p.y);
        atomicAdd(&rho_next[(size_t)c.jc * a.nnx + c.ic], (unsigned long long)(q * c.w00()));
        atomicAdd(&rho_next[(size_t)c.jc * a.nnx + c.ic + 1], (unsigned long long)(q * c.w10()));
        atomicAdd(&rho_next[(size_t)(c.jc + 1) * a.nnx + c.ic], (unsigned long long)(q * c.w01()));
        atomicAdd(&rho_next[(size_t)(c.jc + 1) * a.nnx + c.ic + 1],
                  (unsigned long long)(q * c.w11()));
      } else {
        fl |= CUPIC_FLAG_CAPACITY;
      }
    }
  }
  const unsigned wr = __reduce_add_sync(kFull, nrem);
  if (lane == 0 && wr) atomicAdd(&s_rem, wr);
  fl = __reduce_or_sync(kFull, fl);
  if (lane == 0) raise_flags(ctl, fl);
  __syncthreads();
  for (int k = tid; k < a.ncy; k += kInjBlock)
    if (running[k]) S.cnt[k] = min(S.cnt[k] + running[k], S.cap[k]);
  if (tid == 0 && s_rem) atomicAdd(&ctl->removed[sp], (unsigned long long)s_rem);
}

__global__ void __launch_bounds__(kInjBlock) k_inject_append(SimArgs a) {
  extern __shared__ int running[];
  inject_append(a, blockIdx.x, running);
}

// grid (species, instance)
__global__ void __launch_bounds__(kInjBlock) k_inject_append_batch(const SimArgs *__restrict__ inst) {
  extern __shared__ int running[];
  inject_append(inst[blockIdx.y], blockIdx.x, running);
}

// ---------------------------------------------------------------------------
// end of step: stats ring entry, clocks, charge buffer flip
// ---------------------------------------------------------------------------
__device__ __forceinline__ void finalize(const SimArgs &a) {
  Ctl *ctl = a.ctl;
  if (halted(ctl)) {  // the host completes the halted step and reruns the ones counted here
    if (threadIdx.x == 0) ctl->skipped += 1;
    return;
  }
  __shared__ unsigned long long live[2];
  if (threadIdx.x < 2) live[threadIdx.x] = 0ull;
  __syncthreads();
  // both species' counts in one loop, so each thread's loads of a pass
  // are in flight together
  unsigned long long v0 = 0, v1 = 0;
  for (int k = threadIdx.x; k < a.ncy; k += blockDim.x) {
    v0 += (unsigned long long)a.sp[0].cnt[k];
    v1 += (unsigned long long)a.sp[1].cnt[k];
  }
  for (int o = 16; o > 0; o >>= 1) {
    v0 += __shfl_down_sync(0xffffffffu, v0, o);
    v1 += __shfl_down_sync(0xffffffffu, v1, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&live[0], v0);
    atomicAdd(&live[1], v1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // every field is read before the first store: the ring entry lies in
    // the same block, so interleaved loads and stores would each wait for
    // the one before (one L2 round trip per field)
    const int64_t step = ctl->step;
    const double t = ctl->t;
    const unsigned long long ab0 = ctl->absorbed[0], ab1 = ctl->absorbed[1];
    const unsigned long long rm0 = ctl->removed[0], rm1 = ctl->removed[1];
    const int32_t in0 = ctl->inj_count[0], in1 = ctl->inj_count[1];
    const int32_t sweeps = ctl->sweeps;
    const float residual = ctl->residual;
    const uint32_t sfl = ctl->step_flags, fl = ctl->flags;
    const int32_t cur = ctl->cur;
    cupic_step_stats st{};
    st.step = step;
    st.t = t;
    st.absorbed[0] = (int64_t)ab0;
    st.absorbed[1] = (int64_t)ab1;
    st.removed[0] = (int64_t)rm0;
    st.removed[1] = (int64_t)rm1;
    st.injected[0] = in0;
    st.injected[1] = in1;
    st.live[0] = (int64_t)live[0];
    st.live[1] = (int64_t)live[1];
    st.sweeps = sweeps;
    st.residual = residual;
    st.flags = sfl;
    ctl->ring[step % kStatsRing] = st;
    for (int sp = 0; sp < 2; ++sp) {
      ctl->absorbed[sp] = 0ull;
      ctl->removed[sp] = 0ull;
      ctl->inj_count[sp] = 0;
    }
    ctl->flags = fl | sfl;
    ctl->step_flags = 0u;
    ctl->t = t + a.dt_d;
    ctl->step = step + 1;
    ctl->cur = cur ^ 1;
  }
}

__global__ void k_finalize(SimArgs a) { finalize(a); }

__global__ void k_finalize_batch(const SimArgs *__restrict__ inst) { finalize(inst[blockIdx.x]); }

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------
cudaError_t launch_init_particles(const SimArgs &a, cudaStream_t st) {
  k_init_particles<<<dim3(a.ncy, 2), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_deposit(const SimArgs &a, cudaStream_t st) {
  k_deposit<<<a.ncy, 256, rho_moment_bytes(1, a.ncx), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_zero_next_rho(const SimArgs &a, cudaStream_t st) {
  const size_t n = (size_t)a.nnx * a.nny;
  int blocks = (int)((n + 1023) / 1024);
  if (blocks > 1184) blocks = 1184;
  k_zero_next_rho<<<blocks, 1024, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_uniform_layout(const SpeciesDev &S, int ncy, int capj, cudaStream_t st) {
  k_uniform_layout<<<(ncy + 255) / 256, 256, 0, st>>>(S, ncy, capj);
  return cudaGetLastError();
}

cudaError_t launch_set_time(Ctl *ctl, int64_t step, double t, double tin_e, double tin_i, cudaStream_t st) {
  k_set_time<<<1, 1, 0, st>>>(ctl, step, t, tin_e, tin_i);
  return cudaGetLastError();
}

cudaError_t launch_linear_phi(const SimArgs &a, double phi_p, double *phi64, cudaStream_t st) {
  k_linear_phi<<<dim3((a.nnx + 255) / 256, a.nny), 256, 0, st>>>(a, phi_p, phi64);
  return cudaGetLastError();
}

cudaError_t launch_leapfrog_start(const SimArgs &a, cudaStream_t st) {
  k_leapfrog_start<<<a.ncy, 256, 2 * a.nnx * sizeof(float2), st>>>(a);
  return cudaGetLastError();
}

namespace {
// whether k_push_deposit_narrow fits 4 blocks per SM with `bytes` of
// dynamic shared memory on the current device (cached)
cudaError_t push_narrow(size_t bytes, bool *narrow) {
  static std::mutex mu;
  static std::map<std::pair<int, size_t>, bool> memo;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_pair(dev, bytes);
  const auto it = memo.find(key);
  if (it != memo.end()) {
    *narrow = it->second;
    return cudaSuccess;
  }
  const void *fn = reinterpret_cast<const void *>(k_push_deposit_narrow);
  e = raise_dyn_smem(fn, bytes);
  int n = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_push_deposit_narrow, kPB, bytes);
  if (e != cudaSuccess) return e;
  *narrow = memo[key] = n >= 4;
  return cudaSuccess;
}
}  // namespace

cudaError_t push_set_smem(size_t bytes) {
  bool narrow = false;
  const cudaError_t e = raise_dyn_smem(reinterpret_cast<const void *>(k_push_deposit), bytes);
  return e != cudaSuccess ? e : push_narrow(bytes, &narrow);
}

cudaError_t launch_push_deposit(const SimArgs &a, cudaStream_t st) {
  const size_t sm = push_smem_bytes(a.nnx, kPB);
  bool narrow = false;
  const cudaError_t e = push_narrow(sm, &narrow);
  if (e != cudaSuccess) return e;
  if (narrow)
    k_push_deposit_narrow<<<2 * a.ncy, kPB, sm, st>>>(a);
  else
    k_push_deposit<<<2 * a.ncy, kPB, sm, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_arrive(const SimArgs &a, cudaStream_t st) {
  k_arrive<<<dim3(a.ncy, 2), 128, 0, st>>>(a);
  return cudaGetLastError();
}

// The draws depend only on the clocks and the step's field, so a step can
// run them beside the push; the append needs the push's row counts.
cudaError_t launch_inject_draw(const SimArgs &a, cudaStream_t st) {
  const int cap = max(a.sp[0].inj_cap, a.sp[1].inj_cap);
  k_inject_sched<<<1, 32, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_inject_gen<<<dim3((cap + 127) / 128, 2), 128, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_inject_append(const SimArgs &a, cudaStream_t st) {
  k_inject_append<<<2, kInjBlock, a.ncy * sizeof(int), st>>>(a);
  return cudaGetLastError();
}

template <int PB>
cudaError_t push_batch(const SimArgs *inst, const int2 *row_work, int n, int max_nnx, cudaStream_t st) {
  const size_t sm = push_smem_bytes(max_nnx, PB);
  cudaError_t e = raise_dyn_smem(reinterpret_cast<const void *>(k_push_deposit_batch<PB>), sm);
  if (e != cudaSuccess) return e;
  k_push_deposit_batch<PB><<<2 * n, PB, sm, st>>>(inst, row_work);
  return cudaGetLastError();
}

cudaError_t launch_push_deposit_batch(const SimArgs *inst, const int2 *row_work, int n, int max_nnx,
                                      int threads, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  // 128 threads for rows of up to 64 cells, 512 for longer ones
  return threads == 128 ? push_batch<128>(inst, row_work, n, max_nnx, st)
                        : push_batch<512>(inst, row_work, n, max_nnx, st);
}

cudaError_t launch_arrive_batch(const SimArgs *inst, const int2 *row_work, int n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int ntask = 2 * n;
  k_arrive_batch<<<(ntask + kArriveWarps - 1) / kArriveWarps, 32 * kArriveWarps, 0, st>>>(inst, row_work,
                                                                                        ntask);
  return cudaGetLastError();
}

cudaError_t launch_inject_draw_batch(const SimArgs *inst, int n, int max_inj_cap, cudaStream_t st) {
  k_inject_sched_batch<<<(2 * n + 127) / 128, 128, 0, st>>>(inst, n);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_inject_gen_batch<<<dim3((max_inj_cap + 127) / 128, 2, n), 128, 0, st>>>(inst);
  return cudaGetLastError();
}

cudaError_t launch_inject_append_batch(const SimArgs *inst, int n, int max_ncy, cudaStream_t st) {
  k_inject_append_batch<<<dim3(2, n), kInjBlock, max_ncy * sizeof(int), st>>>(inst);
  return cudaGetLastError();
}

cudaError_t launch_room(const SimArgs &a, cudaStream_t st) {
  k_room<<<2, kRoomBlock, a.ncy * sizeof(int), st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_room_batch(const SimArgs *inst, int n, int max_ncy, cudaStream_t st) {
  k_room_batch<<<dim3(2, n), kRoomBlock, max_ncy * sizeof(int), st>>>(inst);
  return cudaGetLastError();
}

cudaError_t launch_move_rows(const float4 *old, const int64_t *oseg, float4 *parts, const int64_t *nseg,
                             const int32_t *keep, int ncy, cudaStream_t st) {
  k_move_rows<<<ncy, 256, 0, st>>>(old, oseg, parts, nseg, keep);
  return cudaGetLastError();
}

cudaError_t launch_finalize_batch(const SimArgs *inst, int n, cudaStream_t st) {
  k_finalize_batch<<<n, 256, 0, st>>>(inst);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const SimArgs &a, cudaStream_t st) {
  k_finalize<<<1, 1024, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace cupic
