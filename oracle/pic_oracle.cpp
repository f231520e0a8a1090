/*
 * pic_oracle.cpp -- CPU oracle of the cupic per-step PIC cycle.
 *
 * TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py use it to check and time against.  The
 * product path never links it.
 *
 * Parity: pinned.  The input_data normalisation is checked bit for bit
 * against the reference's own init_* getters compiled from its sources
 * (oracle/ref_pin/); the per-kernel arithmetic is checked against analytic
 * known answers (tests/test_oracle.py) because the reference ships no tests
 * or golden vectors.
 *
 * Each stage follows a reference function (file:line in AntonioTejero/cupic)
 * with its intended semantics; the reference defects it does NOT reproduce:
 *   D3  mesh.cu:277-290   volume divide races / divides row 513: here rho =
 *                         sum(q w)/ds^3 with ds^3/2 on both Dirichlet rows.
 *   D4  particles.cu:152  gather uses blockDim.x for the row: here the true
 *                         row index of the particle.
 *   D5  mesh.cu:79-114    in-place (chaotic) Jacobi: here double-buffered.
 *   D7/D8 cc.cu:303-772   nondeterministic bin order: here a stable order.
 *   D10 cc.cu:250-256     injected particles appended to the last bin: here
 *                         to the row their y falls in.
 *   D11 cc.cu:800-804     x<=0 wrap maps 0 to Lx: here [0,Lx).
 *   D15 cc.cu:243-244     injected velocity correction ignores the charge
 *                         sign (wrong for ions): here v += dt' q E/m.
 *
 * Row order after a step (both precisions, and the GPU):
 *   row d = [particles of row d that stayed, in previous order]
 *         + [particles that moved up from row d-1, in previous order]
 *         + [particles that moved down from row d+1, in previous order]
 *         + [injected particles whose y falls in row d, in draw order]
 * A particle that moves more than one row in a step (violating the
 * reference's own one-row assumption, cc.cu:303-636) stays listed in its old
 * row, is deposited at its true position, and raises CUPIC_FLAG_CFL.
 */
#include "pic_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <type_traits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as   */
/* easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies and a      */
/* Weyl-sequence key schedule.                                               */
/* ------------------------------------------------------------------------ */
struct U4 {
  uint32_t v[4];
};

U4 philox(U4 c, uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c.v[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.v[2];
    U4 n;
    n.v[0] = (uint32_t)(p1 >> 32) ^ c.v[1] ^ k0;
    n.v[1] = (uint32_t)p1;
    n.v[2] = (uint32_t)(p0 >> 32) ^ c.v[3] ^ k1;
    n.v[3] = (uint32_t)p0;
    c = n;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

/* uniform on the open interval (0,1), exact in double */
inline double u01(uint32_t r) { return ((double)r + 0.5) * 0x1p-32; }

/* Natural log from IEEE basic operations only (so every IEEE-754 machine
 * gives the same bits): x = m 2^e with m in [sqrt(1/2), sqrt(2)),
 * log m = 2 atanh(s), s = (m-1)/(m+1), by its odd power series to s^23. */
double olog(double x) {
  uint64_t b;
  std::memcpy(&b, &x, 8);
  int e = (int)((b >> 52) & 0x7ff) - 1023;
  b = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull;
  double m;
  std::memcpy(&m, &b, 8);
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

/* sin and cos of theta in [0, pi/4] by Taylor series to the 17th/16th power */
void sincos_small(double th, double *s, double *c) {
  const double t2 = th * th;
  double ps = -1.0 / 355687428096000.0;          /* -1/17! */
  ps = ps * t2 + 1.0 / 1307674368000.0;          /* 1/15! */
  ps = ps * t2 - 1.0 / 6227020800.0;             /* 1/13! */
  ps = ps * t2 + 1.0 / 39916800.0;               /* 1/11! */
  ps = ps * t2 - 1.0 / 362880.0;                 /* 1/9! */
  ps = ps * t2 + 1.0 / 5040.0;                   /* 1/7! */
  ps = ps * t2 - 1.0 / 120.0;                    /* 1/5! */
  ps = ps * t2 + 1.0 / 6.0;                      /* 1/3! */
  *s = th - th * t2 * ps;
  double pc = 1.0 / 20922789888000.0;            /* 1/16! */
  pc = pc * t2 - 1.0 / 87178291200.0;            /* 1/14! */
  pc = pc * t2 + 1.0 / 479001600.0;              /* 1/12! */
  pc = pc * t2 - 1.0 / 3628800.0;                /* 1/10! */
  pc = pc * t2 + 1.0 / 40320.0;                  /* 1/8! */
  pc = pc * t2 - 1.0 / 720.0;                    /* 1/6! */
  pc = pc * t2 + 1.0 / 24.0;                     /* 1/4! */
  pc = pc * t2 - 0.5;                            /* 1/2! */
  *c = 1.0 + t2 * pc;
}

/* sin(2 pi u), cos(2 pi u) for u in [0,1): octant reduction u*8 = o + f */
void osincos2pi(double u, double *s, double *c) {
  const double r = u * 8.0;
  int o = (int)r;
  if (o > 7) o = 7;
  if (o < 0) o = 0;
  const double f = r - (double)o;
  const double qpi = 0.78539816339744831; /* pi/4 */
  double sa, ca;
  if (o & 1) {
    sincos_small((1.0 - f) * qpi, &sa, &ca);
  } else {
    sincos_small(f * qpi, &sa, &ca);
  }
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

/* counter layout of the generator (shared with the GPU build) */
enum { PURPOSE_INIT = 0, PURPOSE_INJECT = 1 };

/* ------------------------------------------------------------------------ */
/* physical constants and input_data parsing (init.cu:424-789, init.h:24-27) */
/* ------------------------------------------------------------------------ */
const double CST_ME = 9.109e-31;
const double CST_E = 1.602e-19;
const double CST_KB = 1.381e-23;
const double CST_EPSILON = 8.854e-12;
const double CST_PI = 3.1415926535897932;

template <class R>
struct P4 {
  R x, y, vx, vy;
};

enum { ROW_ABSORBED = -1, ROW_REMOVED = -2 };

template <class R>
inline R clamp01(R v) {
  return std::fmin(std::fmax(v, (R)0), (R)1);
}

/* floor(v) clamped to [lo,hi]; NaN -> lo */
template <class R>
inline int cfloor(R v, int lo, int hi) {
  if (!(v >= (R)lo)) return lo;
  if (v >= (R)(hi + 1)) return hi;
  int i = (int)std::floor(v);
  return i > hi ? hi : i;
}

template <class R>
struct Sim {
  static constexpr bool F32 = std::is_same<R, float>::value;
  cupic_params p;
  int ncx, ncy, nnx, nny;
  /* constants in the working precision, rounded once from double */
  R ds, inv_ds, Lx, Ly, two_ds, dt, dtqm[2], mhdtqm[2];
  double q[2], m[2], kt[2], dtin[2];
  double cb; /* fixed-point charge -> Jacobi source term, interior rows */
  std::vector<R> phi, ex, ey;
  std::vector<double> phi64; /* F32 with refine_every > 0: the FP64 potential */
  std::vector<int64_t> acc;  /* F32: raw (unfolded) fixed-point charge */
  std::vector<double> accd;  /* F64: raw charge sum */
  bool acc_valid = false;
  std::vector<double> rho_used; /* rho of the last solve */
  std::vector<std::vector<P4<R>>> rows[2];
  int64_t step = 1;
  double t = 0.0;
  double tin[2] = {0.0, 0.0};
  bool tin_set[2] = {false, false};
  cupic_step_stats st;
  uint32_t flags = 0;

  explicit Sim(const cupic_params &pp) : p(pp) {
    ncx = p.ncx;
    ncy = p.ncy;
    nnx = ncx + 1;
    nny = ncy + 1;
    const double Lxd = p.ds * ncx, Lyd = p.ds * ncy;
    ds = (R)p.ds;
    inv_ds = (R)(1.0 / p.ds);
    Lx = (R)Lxd;
    Ly = (R)Lyd;
    two_ds = (R)(2.0 * p.ds);
    dt = (R)p.dt;
    q[0] = p.qe; q[1] = p.qi;
    m[0] = p.me; m[1] = p.mi;
    kt[0] = p.kte; kt[1] = p.kti;
    for (int s = 0; s < 2; ++s) {
      dtqm[s] = (R)(p.dt * q[s] / m[s]);
      mhdtqm[s] = (R)(-0.5 * p.dt * q[s] / m[s]);
    }
    /* init.cu:686-714 */
    dtin[0] = std::sqrt(2.0 * CST_PI * m[0] / kt[0]) / (p.n * Lxd * p.ds);
    dtin[1] = std::sqrt(2.0 * CST_PI * m[1] / kt[1]) / (p.n * Lxd * p.ds);
    cb = std::ldexp(1.0, -32) / (p.ds * p.eps0);
    phi.assign((size_t)nnx * nny, (R)0);
    ex.assign((size_t)nnx * nny, (R)0);
    ey.assign((size_t)nnx * nny, (R)0);
    acc.assign((size_t)nnx * nny, 0);
    accd.assign((size_t)nnx * nny, 0.0);
    rho_used.assign((size_t)nnx * nny, 0.0);
    for (int s = 0; s < 2; ++s) rows[s].assign(ncy, {});
    t = p.n_ini * p.dt + p.dt; /* main.cu:57 */
    step = (int64_t)p.n_ini + 1;
    std::memset(&st, 0, sizeof(st));
  }

  int row_of(R y) const { return cfloor<R>(y * inv_ds, 0, ncy - 1); }

  R wrap(R x) const { /* cc.cu:800-804 with D11 fixed */
    if (x < (R)0) x += Lx;
    if (x >= Lx) x -= Lx;
    return x;
  }

  /* ---- deposition: mesh.cu:196-240 (CIC weights, periodic fold) ---------- */
  template <class F>
  void deposit_one(const P4<R> &a, double qs, F &&sink) const {
    const R sx = a.x * inv_ds;
    const int ic = cfloor<R>(sx, 0, ncx - 1);
    const R fx = clamp01<R>(sx - (R)ic);
    const R sy = a.y * inv_ds;
    const int jc = cfloor<R>(sy, 0, ncy - 1);
    const R fy = clamp01<R>(sy - (R)jc);
    const size_t n00 = (size_t)jc * nnx + ic;
    if constexpr (F32) {
      /* CIC weights in 18-bit fixed point per axis, the cross term FX*FY
       * rounded to a multiple of 2^14; the four sum to 2^32 */
      const int64_t FX = (int64_t)std::rint(fx * 262144.0f);
      const int64_t FY = (int64_t)std::rint(fy * 262144.0f);
      const int64_t W11 = ((FX * FY + 131072) >> 18) << 14;
      const int64_t qq = qs < 0 ? -1 : 1;
      sink(n00, qq * ((int64_t)1 << 32) - qq * ((FX + FY) << 14) + qq * W11);
      sink(n00 + 1, qq * ((FX << 14) - W11));
      sink(n00 + nnx, qq * ((FY << 14) - W11));
      sink(n00 + nnx + 1, qq * W11);
    } else {
      const double gx = 1.0 - fx, gy = 1.0 - fy;
      sink(n00, qs * gx * gy);
      sink(n00 + 1, qs * fx * gy);
      sink(n00 + nnx, qs * gx * fy);
      sink(n00 + nnx + 1, qs * fx * fy);
    }
  }

  void deposit() {
    std::fill(acc.begin(), acc.end(), 0);
    std::fill(accd.begin(), accd.end(), 0.0);
    std::vector<P4<R>> stray[2];
    /* rows of equal parity touch disjoint node rows: two race-free phases */
    for (int phase = 0; phase < 2; ++phase) {
#pragma omp parallel for schedule(dynamic, 4)
      for (int r = phase; r < ncy; r += 2) {
        for (int s = 0; s < 2; ++s) {
          for (const P4<R> &a : rows[s][r]) {
            if (row_of(a.y) != r) continue; /* deposited below */
            if constexpr (F32) {
              deposit_one(a, q[s], [&](size_t n, int64_t w) { acc[n] += w; });
            } else {
              deposit_one(a, q[s], [&](size_t n, double w) { accd[n] += w; });
            }
          }
        }
      }
    }
    for (int s = 0; s < 2; ++s)
      for (int r = 0; r < ncy; ++r)
        for (const P4<R> &a : rows[s][r]) {
          if (row_of(a.y) == r) continue;
          if constexpr (F32) {
            deposit_one(a, q[s], [&](size_t n, int64_t w) { acc[n] += w; });
          } else {
            deposit_one(a, q[s], [&](size_t n, double w) { accd[n] += w; });
          }
        }
    acc_valid = true;
  }

  /* folded charge of node (i,j): the x=0 and x=Lx columns are one node */
  double folded(size_t j, int i) const {
    const size_t r = j * nnx;
    if (i == 0 || i == nnx - 1) {
      return F32 ? (double)(acc[r] + acc[r + nnx - 1]) : accd[r] + accd[r + nnx - 1];
    }
    return F32 ? (double)acc[r + i] : accd[r + i];
  }

  int64_t folded_fixed(size_t j, int i) const {
    const size_t r = j * nnx;
    if (i == 0 || i == nnx - 1) return acc[r] + acc[r + nnx - 1];
    return acc[r + i];
  }

  /* rho = charge / cell volume, ds^3/2 on the Dirichlet rows (D3 fixed) */
  void rho_out(std::vector<double> &out) const {
    out.resize((size_t)nnx * nny);
    const double ds3 = p.ds * p.ds * p.ds;
    const double scale = F32 ? std::ldexp(1.0, -32) : 1.0;
    for (int j = 0; j < nny; ++j) {
      const double vol = (j == 0 || j == nny - 1) ? 0.5 * ds3 : ds3;
      for (int i = 0; i < nnx; ++i) out[(size_t)j * nnx + i] = folded(j, i) * scale / vol;
    }
  }

  bool refined() const { return p.refine_every > 0; }

  /* k fixed Jacobi sweeps of x with source src, the operation order of
   * solve() (no convergence test) */
  void fixed_sweeps(std::vector<R> &x, const std::vector<R> &src, int k) const {
    std::vector<R> nw(x);
    for (int it = 0; it < k; ++it) {
#pragma omp parallel for schedule(static)
      for (int j = 1; j < nny - 1; ++j) {
        const R *c = &x[(size_t)j * nnx];
        const R *dn = c - nnx;
        const R *up = c + nnx;
        const R *bb = &src[(size_t)j * nnx];
        R *o = &nw[(size_t)j * nnx];
        for (int i = 0; i < nnx - 1; ++i) {
          const R W = (i == 0) ? c[nnx - 2] : c[i - 1];
          o[i] = (R)0.25 * ((((bb[i] + W) + c[i + 1]) + up[i]) + dn[i]);
        }
        o[nnx - 1] = o[0];
      }
      x.swap(nw);
    }
  }

  /* Precision form (refine_every = m > 0).  F32: the GPU's algorithm step
   * for step -- FP64 residual r = b - A phi64, m FP32 sweeps on the
   * correction with source (float)r, FP64 update.  F64: plain FP64 Jacobi
   * with the same stop rule (its iterates equal the F32 form's in exact
   * arithmetic).  Stop when max|r| < tol after at least mn sweeps, or at mx
   * sweeps; the residual is checked before every block of m sweeps. */
  void solve_refined(double tol, int mn, int mx, int *sweeps, double *res) {
    const size_t nn = (size_t)nnx * nny;
    const int m = p.refine_every;
    if (F32 && phi64.size() != nn) phi64.assign(phi.begin(), phi.end());
    std::vector<double> b64(nn, 0.0);
    for (int j = 1; j < nny - 1; ++j)
      for (int i = 0; i < nnx; ++i)
        b64[(size_t)j * nnx + i] =
            F32 ? (double)folded_fixed(j, i) * cb : folded(j, i) / (p.ds * p.eps0);
    std::vector<R> rr(nn, (R)0), src;
    if (!F32) src.assign(b64.begin(), b64.end());
    auto P = [&](size_t k) -> double { return F32 ? phi64[k] : (double)phi[k]; };
    int s = 0;
    double rmax = 0.0;
    for (;;) {
      rmax = 0.0;
#pragma omp parallel for reduction(max : rmax) schedule(static)
      for (int j = 1; j < nny - 1; ++j) {
        const size_t rb = (size_t)j * nnx;
        for (int i = 0; i < nnx; ++i) {
          const int ii = i == nnx - 1 ? 0 : i;
          const double c = P(rb + ii), w = P(rb + (ii == 0 ? nnx - 2 : ii - 1));
          const double e = P(rb + ii + 1), n = P(rb + nnx + ii), so = P(rb - nnx + ii);
          const double r = b64[rb + ii] - (4.0 * c - (((w + e) + n) + so));
          rr[rb + i] = (R)r;
          rmax = std::max(rmax, std::fabs(r));
        }
      }
      if ((s >= mn && rmax < tol) || s >= mx) break;
      const int k = std::min(m, mx - s);
      if constexpr (F32) {
        std::vector<R> dl(nn, (R)0);
        fixed_sweeps(dl, rr, k);
        for (int j = 1; j < nny - 1; ++j)
          for (int i = 0; i < nnx; ++i) phi64[(size_t)j * nnx + i] += (double)dl[(size_t)j * nnx + i];
        for (size_t q = 0; q < nn; ++q) phi[q] = (R)phi64[q];
      } else {
        fixed_sweeps(phi, src, k);
      }
      s += k;
    }
    if (sweeps) *sweeps = s;
    if (res) *res = rmax;
    st.sweeps = s;
    st.residual = (float)rmax;
  }

  /* ---- Jacobi: mesh.cu:327-369 (5-point stencil, periodic seam) ---------- */
  void solve(double tol, int min_s, int max_s, int check, int *sweeps, double *res) {
    if (!acc_valid) deposit();
    if (refined()) {
      rho_out(rho_used);
      solve_refined(tol, min_s, max_s, sweeps, res);
      return;
    }
    rho_out(rho_used);
    std::vector<R> b((size_t)nnx * nny, (R)0);
    for (int j = 1; j < nny - 1; ++j)
      for (int i = 0; i < nnx; ++i) {
        if constexpr (F32) {
          b[(size_t)j * nnx + i] = (R)((double)folded_fixed(j, i) * cb);
        } else {
          b[(size_t)j * nnx + i] = folded(j, i) / (p.ds * p.eps0);
        }
      }
    std::vector<R> nw(phi);
    int s = 0;
    double last = std::numeric_limits<double>::infinity();
    if (check < 1) check = 1;
    while (s < max_s) {
      R md = (R)0;
#pragma omp parallel for reduction(max : md) schedule(static)
      for (int j = 1; j < nny - 1; ++j) {
        const R *c = &phi[(size_t)j * nnx];
        const R *dn = c - nnx;
        const R *up = c + nnx;
        const R *bb = &b[(size_t)j * nnx];
        R *o = &nw[(size_t)j * nnx];
        for (int i = 0; i < nnx - 1; ++i) {
          const R W = (i == 0) ? c[nnx - 2] : c[i - 1];
          const R E = c[i + 1];
          const R v = (R)0.25 * ((((bb[i] + W) + E) + up[i]) + dn[i]);
          o[i] = v;
          const R d = std::fabs(v - c[i]);
          if (d > md) md = d;
        }
        o[nnx - 1] = o[0];
        const R d = std::fabs(o[0] - c[nnx - 1]);
        if (d > md) md = d;
      }
      phi.swap(nw);
      ++s;
      if (s % check == 0 || s == max_s) {
        last = (double)md;
        if (s >= min_s && last < tol) break;
      }
    }
    /* keep the Dirichlet rows in both buffers */
    if (sweeps) *sweeps = s;
    if (res) *res = last;
    st.sweeps = s;
    st.residual = (float)last;
  }

  /* ---- field: mesh.cu:413-468 ------------------------------------------ */
  void field() {
    if (F32 && refined()) {  /* from the FP64 potential, rounded once */
      const double ds_d = p.ds;
#pragma omp parallel for schedule(static)
      for (int j = 0; j < nny; ++j)
        for (int i = 0; i < nnx; ++i) {
          const size_t k = (size_t)j * nnx + i, r = (size_t)j * nnx;
          double fx = 0.0, fy;
          if (j == 0) {
            fy = (phi64[k] - phi64[k + nnx]) / ds_d;
          } else if (j == nny - 1) {
            fy = (phi64[k - nnx] - phi64[k]) / ds_d;
          } else {
            const bool seam = i == 0 || i == nnx - 1;
            const double W = seam ? phi64[r + nnx - 2] : phi64[k - 1];
            const double E = seam ? phi64[r + 1] : phi64[k + 1];
            fx = (W - E) / (2.0 * ds_d);
            fy = (phi64[k - nnx] - phi64[k + nnx]) / (2.0 * ds_d);
          }
          ex[k] = (R)fx;
          ey[k] = (R)fy;
        }
      return;
    }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nny; ++j) {
      for (int i = 0; i < nnx; ++i) {
        const size_t k = (size_t)j * nnx + i;
        if (j == 0) {
          ex[k] = (R)0;
          ey[k] = (phi[k] - phi[k + nnx]) / ds;
        } else if (j == nny - 1) {
          ex[k] = (R)0;
          ey[k] = (phi[k - nnx] - phi[k]) / ds;
        } else {
          const size_t r = (size_t)j * nnx;
          const R W = (i == 0 || i == nnx - 1) ? phi[r + nnx - 2] : phi[k - 1];
          const R E = (i == 0 || i == nnx - 1) ? phi[r + 1] : phi[k + 1];
          ex[k] = (W - E) / two_ds;
          ey[k] = (phi[k - nnx] - phi[k + nnx]) / two_ds;
        }
      }
    }
  }

  /* ---- push: particles.cu:145-180 (gather, D4 fixed) + 219-225 (leapfrog),
   *      init.cu:825-826 (leapfrog start), cc.cu:800-804 (wrap) ------------ */
  struct Cls {
    int dest; /* row, ROW_ABSORBED or ROW_REMOVED */
    uint32_t flag;
  };

  void gather(const P4<R> &a, int s, R &Epx, R &Epy) const {
    const R sx = a.x * inv_ds;
    const int ic = cfloor<R>(sx, 0, ncx - 1);
    const R fx = clamp01<R>(sx - (R)ic);
    const R fy = clamp01<R>(a.y * inv_ds - (R)s);
    const R gx = (R)1 - fx, gy = (R)1 - fy;
    const R w00 = gx * gy, w10 = fx * gy, w01 = gx * fy, w11 = fx * fy;
    const size_t b = (size_t)s * nnx + ic;
    Epx = w00 * ex[b];
    Epx = std::fma(w10, ex[b + 1], Epx);
    Epx = std::fma(w01, ex[b + nnx], Epx);
    Epx = std::fma(w11, ex[b + nnx + 1], Epx);
    Epy = w00 * ey[b];
    Epy = std::fma(w10, ey[b + 1], Epy);
    Epy = std::fma(w01, ey[b + nnx], Epy);
    Epy = std::fma(w11, ey[b + nnx + 1], Epy);
  }

  Cls classify(const P4<R> &a, int s) const {
    if (!std::isfinite(a.x) || !std::isfinite(a.y) || !std::isfinite(a.vx) ||
        !std::isfinite(a.vy))
      return {ROW_REMOVED, CUPIC_FLAG_NONFINITE};
    if (a.y < (R)0) return {ROW_ABSORBED, 0};
    if (a.y >= Ly) return {ROW_REMOVED, 0};
    uint32_t f = 0;
    if (a.x < (R)0 || a.x >= Lx) f |= CUPIC_FLAG_XRANGE;
    const int d = row_of(a.y);
    if (s >= 0 && (d > s + 1 || d < s - 1)) return {s, f | CUPIC_FLAG_CFL};
    return {d, f};
  }

  void push(int mode) {
    for (int sp = 0; sp < 2; ++sp) {
      auto &R_ = rows[sp];
      if (mode == 1) {
#pragma omp parallel for schedule(dynamic, 4)
        for (int r = 0; r < ncy; ++r)
          for (P4<R> &a : R_[r]) {
            R Ex, Ey;
            gather(a, r, Ex, Ey);
            a.vx = std::fma(mhdtqm[sp], Ex, a.vx);
            a.vy = std::fma(mhdtqm[sp], Ey, a.vy);
          }
        continue;
      }
      std::vector<std::vector<P4<R>>> stay(ncy), up(ncy), down(ncy);
      std::vector<int64_t> nabs(ncy, 0), nrem(ncy, 0);
      std::vector<uint32_t> fl(ncy, 0);
#pragma omp parallel for schedule(dynamic, 4)
      for (int r = 0; r < ncy; ++r) {
        for (P4<R> a : R_[r]) {
          R Ex, Ey;
          gather(a, r, Ex, Ey);
          a.vx = std::fma(dtqm[sp], Ex, a.vx);
          a.vy = std::fma(dtqm[sp], Ey, a.vy);
          a.x = std::fma(dt, a.vx, a.x);
          a.y = std::fma(dt, a.vy, a.y);
          a.x = wrap(a.x);
          const Cls c = classify(a, r);
          fl[r] |= c.flag;
          if (c.dest == ROW_ABSORBED) {
            nabs[r]++;
          } else if (c.dest == ROW_REMOVED) {
            nrem[r]++;
          } else if (c.dest == r) {
            stay[r].push_back(a);
          } else if (c.dest == r + 1) {
            up[r].push_back(a);
          } else {
            down[r].push_back(a);
          }
        }
      }
      int64_t ta = 0, tr = 0;
      for (int r = 0; r < ncy; ++r) {
        ta += nabs[r];
        tr += nrem[r];
        flags |= fl[r];
        st.flags |= fl[r];
      }
      for (int d = 0; d < ncy; ++d) {
        std::vector<P4<R>> &o = stay[d];
        if (d > 0) o.insert(o.end(), up[d - 1].begin(), up[d - 1].end());
        if (d + 1 < ncy) o.insert(o.end(), down[d + 1].begin(), down[d + 1].end());
        R_[d].swap(o);
      }
      st.absorbed[sp] = ta;
      st.removed[sp] = tr;
    }
    acc_valid = false;
  }

  /* ---- injection: cc.cu:179-256 ---------------------------------------- */
  void inject(double tnow) {
    const double fpt = tnow + p.dt, fvt = tnow + 0.5 * p.dt; /* cc.cu:147-148 */
    const uint32_t k0 = (uint32_t)p.seed, k1 = (uint32_t)(p.seed >> 32);
    const double Lxd = p.ds * ncx, Lyd = p.ds * ncy, inv_dsd = 1.0 / p.ds;
    const size_t top = (size_t)(nny - 1) * nnx;
    for (int sp = 0; sp < 2; ++sp) {
      if (!tin_set[sp]) { /* cc.cu:35-36 static initialisation */
        tin[sp] = tnow + dtin[sp];
        tin_set[sp] = true;
      }
      int in = 0;
      if (tin[sp] < fpt) in = 1 + (int)((fpt - tin[sp]) / dtin[sp]); /* cc.cu:179 */
      const double sig = std::sqrt(kt[sp] / m[sp]);
      const double qm = q[sp] / m[sp];
      std::vector<std::vector<P4<R>>> add(ncy);
      int64_t rem = 0;
      for (int k = 0; k < in; ++k) {
        U4 c = {{(uint32_t)k, (uint32_t)step, (uint32_t)((uint64_t)step >> 32),
                 (uint32_t)((PURPOSE_INJECT << 8) | sp)}};
        U4 r = philox(c, k0, k1);
        double x = u01(r.v[0]) * Lxd;
        double cs, sn;
        osincos2pi(u01(r.v[2]), &sn, &cs);
        double vx = sig * (std::sqrt(-2.0 * olog(u01(r.v[1]))) * cs);
        double vy = -(sig * std::sqrt(-2.0 * olog(u01(r.v[3]))));
        /* field at the injection point (x, Ly): top node row */
        int ic = cfloor<double>(x * inv_dsd, 0, ncx - 1);
        double fx = clamp01<double>(x * inv_dsd - (double)ic);
        const double Epx = (1.0 - fx) * (double)ex[top + ic] + fx * (double)ex[top + ic + 1];
        const double Epy = (1.0 - fx) * (double)ey[top + ic] + fx * (double)ey[top + ic + 1];
        const double dp = fpt - tin[sp], dv = fvt - tin[sp];
        x = x + dp * vx;
        double y = Lyd + dp * vy;
        vx = vx + dv * (qm * Epx);
        vy = vy + dv * (qm * Epy);
        tin[sp] += dtin[sp];
        P4<R> a = {(R)x, (R)y, (R)vx, (R)vy};
        a.x = wrap(a.x);
        const Cls cl = classify(a, -1);
        flags |= cl.flag;
        st.flags |= cl.flag;
        if (cl.dest < 0) {
          rem++;
          continue;
        }
        add[cl.dest].push_back(a);
      }
      for (int d = 0; d < ncy; ++d)
        rows[sp][d].insert(rows[sp][d].end(), add[d].begin(), add[d].end());
      st.injected[sp] = in;
      st.removed[sp] += rem;
    }
    acc_valid = false;
  }

  /* ---- initial plasma: init.cu:159-179 (own seeded generator), 235-241 ---- */
  void init_plasma() {
    const uint32_t k0 = (uint32_t)p.seed, k1 = (uint32_t)(p.seed >> 32);
    const double Lxd = p.ds * ncx;
    for (int sp = 0; sp < 2; ++sp) {
      const double sig = std::sqrt(kt[sp] / m[sp]);
#pragma omp parallel for schedule(dynamic, 4)
      for (int j = 0; j < ncy; ++j) {
        std::vector<P4<R>> &o = rows[sp][j];
        o.resize(p.ppr);
        for (int k = 0; k < p.ppr; ++k) {
          U4 c = {{(uint32_t)k, (uint32_t)j, 0u, (uint32_t)((PURPOSE_INIT << 8) | sp)}};
          U4 r = philox(c, k0, k1);
          const double x = u01(r.v[0]) * Lxd;
          const double y = ((double)j + u01(r.v[1])) * p.ds;
          const double rr = std::sqrt(-2.0 * olog(u01(r.v[2])));
          double sn, cs;
          osincos2pi(u01(r.v[3]), &sn, &cs);
          P4<R> a = {(R)x, (R)y, (R)(sig * (rr * cs)), (R)(sig * (rr * sn))};
          a.x = wrap(a.x);
          for (int it = 0; it < 16 && row_of(a.y) > j; ++it)
            a.y = std::nextafter(a.y, (R)0);
          for (int it = 0; it < 16 && row_of(a.y) < j; ++it)
            a.y = std::nextafter(a.y, Ly);
          o[k] = a;
        }
      }
    }
    if (F32 && refined()) phi64.assign((size_t)nnx * nny, 0.0);
    for (int j = 0; j < nny; ++j)
      for (int i = 0; i < nnx; ++i) {
        const double v = (1.0 - (double)j / (double)ncy) * p.phi_p;
        phi[(size_t)j * nnx + i] = (R)v;
        if (F32 && refined()) phi64[(size_t)j * nnx + i] = v;
      }
    deposit();
    solve(p.init_tol, p.init_min_sweeps, p.init_max_sweeps, p.check_every, nullptr, nullptr);
    field();
    push(1);
    t = p.n_ini * p.dt + p.dt;
    step = (int64_t)p.n_ini + 1;
    tin_set[0] = tin_set[1] = false;
  }

  void step_once() {
    std::memset(&st, 0, sizeof(st));
    st.step = step;
    st.t = t;
    solve(p.tol, p.min_sweeps, p.max_sweeps, p.check_every, nullptr, nullptr);
    field();
    push(0);
    inject(t);
    deposit();
    int64_t ne = 0, ni = 0;
    for (int r = 0; r < ncy; ++r) {
      ne += (int64_t)rows[0][r].size();
      ni += (int64_t)rows[1][r].size();
    }
    st.live[0] = ne;
    st.live[1] = ni;
    t += p.dt;
    step++;
  }

  int load(int sp, const double *xyvv, int64_t n) {
    std::vector<std::vector<P4<R>>> nr(ncy);
    for (int64_t k = 0; k < n; ++k) {
      P4<R> a = {(R)xyvv[4 * k], (R)xyvv[4 * k + 1], (R)xyvv[4 * k + 2], (R)xyvv[4 * k + 3]};
      if (!(a.x >= (R)0 && a.x < Lx && a.y >= (R)0 && a.y < Ly)) return CUPIC_ERR_ARG;
      nr[row_of(a.y)].push_back(a);
    }
    rows[sp].swap(nr);
    acc_valid = false;
    return CUPIC_OK;
  }
};

struct Handle {
  int fp64;
  Sim<float> *f;
  Sim<double> *d;
};

template <class Fn>
int dispatch(void *h, Fn &&fn) {
  Handle *H = (Handle *)h;
  if (!H) return CUPIC_ERR_ARG;
  if (H->fp64) return fn(*H->d);
  return fn(*H->f);
}

/* read line n after the header of an input_data file (init.cu:424-447) */
bool read_line(const char *path, int n, char *line, size_t cap) {
  FILE *f = std::fopen(path, "r");
  if (!f) return false;
  bool ok = std::fgets(line, (int)cap, f) != nullptr; /* header */
  for (int i = 0; ok && i < n; ++i) ok = std::fgets(line, (int)cap, f) != nullptr;
  std::fclose(f);
  return ok;
}

bool read_double(const char *path, int n, double *v) {
  char line[256];
  return read_line(path, n, line, sizeof line) && std::sscanf(line, "%*s = %lf;", v) == 1;
}

bool read_int(const char *path, int n, int *v) {
  char line[256];
  return read_line(path, n, line, sizeof line) && std::sscanf(line, "%*s = %d;", v) == 1;
}

void finalize(cupic_params *p) {
  const double Lx = p->ds * p->ncx;
  p->ppr = (int32_t)(p->n * Lx * p->ds * p->ds); /* init.cu:136 */
}

} /* namespace */

extern "C" {

void ora_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  U4 c = {{ctr[0], ctr[1], ctr[2], ctr[3]}};
  U4 r = philox(c, key[0], key[1]);
  for (int i = 0; i < 4; ++i) out[i] = r.v[i];
}

double ora_log(double x) { return olog(x); }
void ora_sincos2pi(double u, double *s, double *c) { osincos2pi(u, s, c); }

void ora_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int ora_params_default(cupic_params *p) {
  if (!p) return CUPIC_ERR_ARG;
  std::memset(p, 0, sizeof(*p));
  p->ncx = 64;
  p->ncy = 256;
  p->ds = 0.5;
  p->dt = 0.05;
  p->n = 160.0;
  p->eps0 = 160.0;
  p->phi_p = -5.0;
  p->me = 1.0;
  p->mi = 100.0;
  p->kte = 1.0;
  p->kti = 1.0;
  p->qe = -1.0;
  p->qi = 1.0;
  p->tol = 1e-6;
  p->min_sweeps = 1;
  p->max_sweeps = 2000;
  p->check_every = 1;
  p->init_tol = 1e-3;
  p->init_min_sweeps = 1;
  p->init_max_sweeps = 2000;
  p->n_ini = 0;
  p->n_prev = 0;
  p->n_save = 100;
  p->n_fin = 1000;
  p->row_slack = 0.5;
  p->stage_frac = 0.25;
  p->seed = 0;
  finalize(p);
  return CUPIC_OK;
}

/* restatement of read_input_file + init_* getters (init.cu:424-789) */
int ora_params_from_input_data(const char *path, cupic_params *p) {
  if (!path || !p) return CUPIC_ERR_ARG;
  ora_params_default(p);
  int n_ini, n_prev, n_save, n_fin, ncx, ncy;
  double ne, Te, beta, gamma, phi_p, ds, dt;
  if (!read_int(path, 1, &n_ini) || !read_int(path, 2, &n_prev) || !read_int(path, 3, &n_save) ||
      !read_int(path, 4, &n_fin) || !read_double(path, 5, &ne) || !read_double(path, 6, &Te) ||
      !read_double(path, 7, &beta) || !read_double(path, 8, &gamma) ||
      !read_double(path, 9, &phi_p) || !read_int(path, 10, &ncx) || !read_int(path, 11, &ncy) ||
      !read_double(path, 12, &ds) || !read_double(path, 13, &dt))
    return CUPIC_ERR_IO;
  const double Dl = std::sqrt(CST_EPSILON * CST_KB * Te / (ne * CST_E * CST_E)); /* :729 */
  double n = ne;
  n *= Dl * Dl * Dl; /* :552 */
  double eps = CST_EPSILON; /* :622-626 */
  eps /= std::pow(Dl * std::sqrt(CST_ME / (CST_KB * Te)), 2);
  eps /= CST_E * CST_E;
  eps *= Dl * Dl * Dl;
  eps *= CST_ME;
  double php = phi_p;
  php *= CST_E / (CST_KB * Te); /* :534 */
  p->n_ini = n_ini;
  p->n_prev = n_prev;
  p->n_save = n_save;
  p->n_fin = n_fin;
  p->ncx = ncx;
  p->ncy = ncy;
  p->ds = ds;
  p->dt = dt;
  p->n = n;
  p->eps0 = eps;
  p->phi_p = php;
  p->mi = gamma;
  p->kti = beta;
  /* main.cu:64 and init.cu:254 with mesh.cu:67,94 */
  const int mn = std::max(ncx + 1, ncy + 1) + 1;
  p->tol = 1e-4;
  p->min_sweeps = mn;
  p->max_sweeps = 1000000;
  p->check_every = 1;
  p->init_tol = 1e-3;
  p->init_min_sweeps = mn;
  p->init_max_sweeps = 1000000;
  finalize(p);
  return CUPIC_OK;
}

void *ora_create(const cupic_params *p, int fp64) {
  if (!p || p->ncx < 2 || p->ncy < 2 || !(p->ds > 0) || !(p->dt > 0)) return nullptr;
  Handle *h = new Handle{fp64, nullptr, nullptr};
  if (fp64)
    h->d = new Sim<double>(*p);
  else
    h->f = new Sim<float>(*p);
  return h;
}

void ora_destroy(void *h) {
  Handle *H = (Handle *)h;
  if (!H) return;
  delete H->f;
  delete H->d;
  delete H;
}

int ora_init_plasma(void *h) {
  return dispatch(h, [](auto &s) { s.init_plasma(); return (int)CUPIC_OK; });
}

int ora_load(void *h, int sp, const double *xyvv, int64_t n) {
  if (sp < 0 || sp > 1 || n < 0 || (n > 0 && !xyvv)) return CUPIC_ERR_ARG;
  return dispatch(h, [&](auto &s) { return s.load(sp, xyvv, n); });
}

int ora_set_time(void *h, int64_t step, double t, double tin_e, double tin_i) {
  return dispatch(h, [&](auto &s) {
    s.step = step;
    s.t = t;
    s.tin[0] = tin_e;
    s.tin[1] = tin_i;
    s.tin_set[0] = tin_e >= 0;
    s.tin_set[1] = tin_i >= 0;
    return (int)CUPIC_OK;
  });
}

int ora_get_time(void *h, int64_t *step, double *t, double *tin_e, double *tin_i) {
  return dispatch(h, [&](auto &s) {
    if (step) *step = s.step;
    if (t) *t = s.t;
    if (tin_e) *tin_e = s.tin_set[0] ? s.tin[0] : -1.0;
    if (tin_i) *tin_i = s.tin_set[1] ? s.tin[1] : -1.0;
    return (int)CUPIC_OK;
  });
}

int ora_deposit(void *h) {
  return dispatch(h, [](auto &s) { s.deposit(); return (int)CUPIC_OK; });
}

int ora_solve(void *h, double tol, int32_t min_s, int32_t max_s, int32_t check, int32_t *sweeps,
              double *res) {
  return dispatch(h, [&](auto &s) {
    int sw = 0;
    s.solve(tol, min_s, max_s, check, &sw, res);
    if (sweeps) *sweeps = sw;
    return (int)CUPIC_OK;
  });
}

int ora_field(void *h) {
  return dispatch(h, [](auto &s) { s.field(); return (int)CUPIC_OK; });
}

int ora_push(void *h, int mode) {
  return dispatch(h, [&](auto &s) { s.push(mode); return (int)CUPIC_OK; });
}

int ora_inject(void *h, double t) {
  return dispatch(h, [&](auto &s) { s.inject(t); return (int)CUPIC_OK; });
}

int ora_step(void *h, int32_t n) {
  return dispatch(h, [&](auto &s) {
    for (int i = 0; i < n; ++i) s.step_once();
    return (int)CUPIC_OK;
  });
}

int ora_get_counts(void *h, int64_t *ne, int64_t *ni) {
  return dispatch(h, [&](auto &s) {
    int64_t a = 0, b = 0;
    for (int r = 0; r < s.ncy; ++r) {
      a += (int64_t)s.rows[0][r].size();
      b += (int64_t)s.rows[1][r].size();
    }
    if (ne) *ne = a;
    if (ni) *ni = b;
    return (int)CUPIC_OK;
  });
}

int ora_get_particles(void *h, int sp, double *out) {
  if (sp < 0 || sp > 1 || !out) return CUPIC_ERR_ARG;
  return dispatch(h, [&](auto &s) {
    size_t k = 0;
    for (int r = 0; r < s.ncy; ++r)
      for (const auto &a : s.rows[sp][r]) {
        out[k++] = (double)a.x;
        out[k++] = (double)a.y;
        out[k++] = (double)a.vx;
        out[k++] = (double)a.vy;
      }
    return (int)CUPIC_OK;
  });
}

/* the push's CIC field gather (particles.cu:145-180, D4 fixed) at every
 * particle of a species, in row order */
int ora_gather(void *h, int sp, double *ex, double *ey) {
  if (sp < 0 || sp > 1 || !ex || !ey) return CUPIC_ERR_ARG;
  return dispatch(h, [&](auto &s) {
    size_t k = 0;
    for (int r = 0; r < s.ncy; ++r)
      for (const auto &a : s.rows[sp][r]) {
        decltype(a.x) gx, gy;
        s.gather(a, r, gx, gy);
        ex[k] = (double)gx;
        ey[k++] = (double)gy;
      }
    return (int)CUPIC_OK;
  });
}

int ora_get_row_counts(void *h, int sp, int32_t *counts) {
  if (sp < 0 || sp > 1 || !counts) return CUPIC_ERR_ARG;
  return dispatch(h, [&](auto &s) {
    for (int r = 0; r < s.ncy; ++r) counts[r] = (int32_t)s.rows[sp][r].size();
    return (int)CUPIC_OK;
  });
}

int ora_get_phi(void *h, double *o) {
  return dispatch(h, [&](auto &s) {
    if (!s.phi64.empty()) {  // the precision form's FP64 potential
      for (size_t k = 0; k < s.phi64.size(); ++k) o[k] = s.phi64[k];
      return (int)CUPIC_OK;
    }
    for (size_t k = 0; k < s.phi.size(); ++k) o[k] = (double)s.phi[k];
    return (int)CUPIC_OK;
  });
}

int ora_set_phi(void *h, const double *v) {
  return dispatch(h, [&](auto &s) {
    using R = typename std::decay<decltype(s.phi[0])>::type;
    for (size_t k = 0; k < s.phi.size(); ++k) s.phi[k] = (R)v[k];
    if (s.F32 && s.refined()) s.phi64.assign(v, v + s.phi.size());
    return (int)CUPIC_OK;
  });
}

int ora_get_field(void *h, double *ex, double *ey) {
  return dispatch(h, [&](auto &s) {
    for (size_t k = 0; k < s.ex.size(); ++k) {
      ex[k] = (double)s.ex[k];
      ey[k] = (double)s.ey[k];
    }
    return (int)CUPIC_OK;
  });
}

int ora_get_rho(void *h, int which, double *o) {
  return dispatch(h, [&](auto &s) {
    if (which == 1) {
      std::copy(s.rho_used.begin(), s.rho_used.end(), o);
      return (int)CUPIC_OK;
    }
    if (!s.acc_valid) s.deposit();
    std::vector<double> r;
    s.rho_out(r);
    std::copy(r.begin(), r.end(), o);
    return (int)CUPIC_OK;
  });
}

int ora_get_rho_fixed(void *h, int64_t *o) {
  Handle *H = (Handle *)h;
  if (!H || H->fp64) return CUPIC_ERR_ARG;
  if (!H->f->acc_valid) H->f->deposit();
  std::copy(H->f->acc.begin(), H->f->acc.end(), o);
  return CUPIC_OK;
}

int ora_get_stats(void *h, cupic_step_stats *st) {
  return dispatch(h, [&](auto &s) {
    *st = s.st;
    return (int)CUPIC_OK;
  });
}

uint32_t ora_get_flags(void *h) {
  Handle *H = (Handle *)h;
  if (!H) return 0;
  return H->fp64 ? H->d->flags : H->f->flags;
}

} /* extern "C" */
