// io.cu -- host-format particle upload/download on the device.
//
// Upload (read_particle_file, init.cu:348-420): the caller's array of the
// reference's particle struct (4 doubles x,y,vx,vy per particle, any order)
// is copied to the device once, converted to float4, and binned by y row
// with a stable counting sort: per-chunk row histograms, a per-row scan over
// chunks, then a scatter that ranks equal rows in input order.
// Download (particles_snapshot, diagnostic.cu:48-87): rows are packed in row
// order into one buffer and copied out with a single transfer.
#include "cupic_internal.cuh"
#include "kernels.h"

namespace cupic {

namespace {
constexpr int kLoadBlock = 1024;
constexpr unsigned kFull = 0xffffffffu;
}  // namespace

// convert + validate + per-chunk row histogram
__global__ void __launch_bounds__(kLoadBlock)
    k_load_hist(SimArgs a, const double *in, int64_t n, int64_t chunk, float4 *tmp, int32_t *H,
                unsigned *bad) {
  extern __shared__ int hist[];
  const int b = blockIdx.x;
  for (int j = threadIdx.x; j < a.ncy; j += kLoadBlock) hist[j] = 0;
  __syncthreads();
  const int64_t k0 = (int64_t)b * chunk, k1 = min(n, k0 + chunk);
  unsigned nbad = 0;
  for (int64_t k = k0 + threadIdx.x; k < k1; k += kLoadBlock) {
    const double2 xy = reinterpret_cast<const double2 *>(in)[2 * k];
    const double2 vv = reinterpret_cast<const double2 *>(in)[2 * k + 1];
    const float4 p = make_float4((float)xy.x, (float)xy.y, (float)vv.x, (float)vv.y);
    tmp[k] = p;
    if (!(p.x >= 0.0f && p.x < a.Lx && p.y >= 0.0f && p.y < a.Ly)) {
      ++nbad;
      continue;
    }
    atomicAdd(&hist[row_of(a, p.y)], 1);
  }
  if (nbad) atomicAdd(bad, nbad);
  __syncthreads();
  for (int j = threadIdx.x; j < a.ncy; j += kLoadBlock) H[(size_t)b * a.ncy + j] = hist[j];
}

// per-row exclusive scan over chunks; row totals
__global__ void k_load_scan(int32_t *H, int nb, int ncy, int32_t *cnt) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ncy) return;
  int s = 0;
  for (int b = 0; b < nb; ++b) {
    const int v = H[(size_t)b * ncy + j];
    H[(size_t)b * ncy + j] = s;
    s += v;
  }
  cnt[j] = s;
}

// stable scatter into the row segments
__global__ void __launch_bounds__(kLoadBlock)
    k_load_scatter(SimArgs a, int sp, const float4 *tmp, int64_t n, int64_t chunk,
                   const int32_t *H) {
  extern __shared__ int running[];
  constexpr int NW = kLoadBlock / 32;
  const int b = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const SpeciesDev &S = a.sp[sp];
  for (int j = threadIdx.x; j < a.ncy; j += kLoadBlock) running[j] = H[(size_t)b * a.ncy + j];
  __syncthreads();
  const int64_t k0 = (int64_t)b * chunk, k1 = min(n, k0 + chunk);
  for (int64_t base = k0; base < k1; base += kLoadBlock) {
    const int64_t k = base + threadIdx.x;
    int d = -1;
    float4 p;
    if (k < k1) {
      p = tmp[k];
      d = row_of(a, p.y);
    }
    const int key = d >= 0 ? d : -1 - lane;
    const uint32_t grp = __match_any_sync(kFull, key);
    const int leader = __ffs(grp) - 1;
    const int rank = __popc(grp & ((1u << lane) - 1u));
    int bv = 0;
    for (int w = 0; w < NW; ++w) {
      if (warp == w && d >= 0 && lane == leader) {
        bv = running[d];
        running[d] = bv + __popc(grp);
      }
      __syncthreads();
    }
    const int b0 = __shfl_sync(kFull, bv, leader);
    if (d >= 0) S.parts[S.seg[d] + b0 + rank] = p;
  }
}

// rows -> packed array in row order (f32 or the reference's f64 struct)
__global__ void k_pack_rows(SimArgs a, int sp, const int64_t *off, float4 *out32, double *out64) {
  const int j = blockIdx.x;
  const SpeciesDev &S = a.sp[sp];
  const float4 *row = S.parts + S.seg[j];
  const int64_t o = off[j];
  const int n = S.cnt[j];
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const float4 p = row[k];
    if (out32) out32[o + k] = p;
    if (out64) {
      double2 *q = reinterpret_cast<double2 *>(out64) + 2 * (o + k);
      q[0] = make_double2(p.x, p.y);
      q[1] = make_double2(p.z, p.w);
    }
  }
}

int load_blocks(int64_t n, int num_sms) {
  int64_t nb = (n + 8191) / 8192;
  if (nb > 4 * num_sms) nb = 4 * num_sms;
  return nb < 1 ? 1 : (int)nb;
}

cudaError_t launch_load_hist(const SimArgs &a, const double *in, int64_t n, int nb, float4 *tmp,
                             int32_t *H, unsigned *bad, cudaStream_t st) {
  const int64_t chunk = (n + nb - 1) / nb;
  k_load_hist<<<nb, kLoadBlock, a.ncy * sizeof(int), st>>>(a, in, n, chunk, tmp, H, bad);
  return cudaGetLastError();
}

cudaError_t launch_load_scan(int32_t *H, int nb, int ncy, int32_t *cnt, cudaStream_t st) {
  k_load_scan<<<(ncy + 255) / 256, 256, 0, st>>>(H, nb, ncy, cnt);
  return cudaGetLastError();
}

cudaError_t launch_load_scatter(const SimArgs &a, int sp, const float4 *tmp, int64_t n, int nb,
                                const int32_t *H, cudaStream_t st) {
  const int64_t chunk = (n + nb - 1) / nb;
  k_load_scatter<<<nb, kLoadBlock, a.ncy * sizeof(int), st>>>(a, sp, tmp, n, chunk, H);
  return cudaGetLastError();
}

cudaError_t launch_pack_rows(const SimArgs &a, int sp, const int64_t *off, float4 *out32,
                             double *out64, cudaStream_t st) {
  k_pack_rows<<<a.ncy, 256, 0, st>>>(a, sp, off, out32, out64);
  return cudaGetLastError();
}

}  // namespace cupic
