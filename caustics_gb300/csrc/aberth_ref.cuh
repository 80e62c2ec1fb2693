// FP64 Ehrlich-Aberth iteration with the reference's operation order and
// rounding (lib/ehrlich_aberth/ehrlich_aberth.h:60-150, horner.h:219-267,
// init_est.h:57-102): products and sums rounded one by one (no FMA
// contraction), Smith's complex division, hypot for |z|, z^2 = exp(2 log z) in
// the reversed correction, and the reference's real-valued initial guesses.
//
// It is used only where the reference's *labelling* of roots matters and is
// decided by the iteration's dynamics: the first limb point's cold start and the
// few warm-started limb steps whose nearest-root map is ambiguous.  The roots
// themselves always come from the fast solvers in aberth.cuh.
#pragma once
#include "cplx.cuh"

namespace refea {

__device__ __forceinline__ cd mul(cd a, cd b) {
  return cd{__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x))};
}
__device__ __forceinline__ cd add(cd a, cd b) { return cd{__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y)}; }
__device__ __forceinline__ cd sub(cd a, cd b) { return cd{__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y)}; }
__device__ __forceinline__ cd scale(cd a, double s) { return cd{__dmul_rn(a.x, s), __dmul_rn(a.y, s)}; }
__device__ __forceinline__ double absc(cd a) { return hypot(a.x, a.y); }
__device__ __forceinline__ cd div(cd a, cd b) {
  if (fabs(b.x) >= fabs(b.y)) {
    double r = __ddiv_rn(b.y, b.x), d = __dadd_rn(b.x, __dmul_rn(b.y, r));
    return cd{__ddiv_rn(__dadd_rn(a.x, __dmul_rn(a.y, r)), d), __ddiv_rn(__dsub_rn(a.y, __dmul_rn(a.x, r)), d)};
  }
  double r = __ddiv_rn(b.x, b.y), d = __dadd_rn(__dmul_rn(b.x, r), b.y);
  return cd{__ddiv_rn(__dadd_rn(__dmul_rn(a.x, r), a.y), d), __ddiv_rn(__dsub_rn(__dmul_rn(a.y, r), a.x), d)};
}
__device__ __forceinline__ cd recip(cd b) { return div(cd{1.0, 0.0}, b); }
__device__ __forceinline__ cd sq_pow(cd z) {
  double m = exp(__dmul_rn(2.0, log(absc(z)))), t = __dmul_rn(2.0, atan2(z.y, z.x));
  return cd{__dmul_rn(m, cos(t)), __dmul_rn(m, sin(t))};
}

template <int DEG>
__device__ void init_real(const double (&alpha)[DEG + 1], cd (&z)[DEG]) {
  int hx[DEG + 1];
  double hy[DEG + 1];
  int k = 0;
  for (int i = DEG; i >= 0; --i) {
    double y = alpha[i] > 0 ? log(alpha[i]) : -1e30;
    while (k >= 2) {
      double ccw = __dsub_rn(__dmul_rn((double)(hx[k - 1] - hx[k - 2]), __dsub_rn(y, hy[k - 2])),
                             __dmul_rn(__dsub_rn(hy[k - 1], hy[k - 2]), (double)(i - hx[k - 2])));
      if (ccw <= 0) --k; else break;
    }
    hx[k] = i;
    hy[k] = y;
    ++k;
  }
  cd t[DEG];
  const double pi2 = 6.28318530717958647693, th = __ddiv_rn(pi2, (double)DEG);
  int n = 0;
  for (int i = k - 2; i >= 0; --i) {
    int nz = hx[i] - hx[i + 1];
    double r = __ddiv_rn(pow(alpha[hx[i + 1]], __ddiv_rn(1.0, (double)nz)), pow(alpha[hx[i]], __ddiv_rn(1.0, (double)nz)));
    double ang = __ddiv_rn(pi2, (double)nz);
    for (int j = 0; j < nz && n + j < DEG; ++j) {
      double phi = __dadd_rn(__dadd_rn(__dmul_rn(ang, (double)j), __dmul_rn(th, (double)i)), 0.7);
      t[n + j] = cd{__dmul_rn(r, sin(phi)), 0.0};
    }
    n += nz;
  }
#pragma unroll
  for (int i = 0; i < DEG; ++i) z[i] = t[i];
}

// Returns the iteration count, -1 if itmax was reached.
template <int DEG>
__device__ int solve(const cd (&p)[DEG + 1], cd (&z)[DEG], int itmax, bool warm) {
  double alpha[DEG + 1];
#pragma unroll
  for (int i = 0; i <= DEG; ++i) alpha[i] = absc(p[i]);
  if (!warm) init_real<DEG>(alpha, z);
#pragma unroll
  for (int i = 0; i <= DEG; ++i) alpha[i] = __dmul_rn(alpha[i], fma(3.8284271247461900976, (double)i, 1.0));
  uint32_t conv = 0;
  const uint32_t all = (1u << DEG) - 1u;
  const double EPS = 1.1102230246251565e-16;
  for (int it = 0; it < itmax; ++it) {
#pragma unroll
    for (int j = 0; j < DEG; ++j) {
      if ((conv >> j) & 1u) continue;
      double az = absc(z[j]);
      bool rev = az > 1.0;
      cd x = rev ? recip(z[j]) : z[j];
      double ax = rev ? __ddiv_rn(1.0, az) : az;
      double b = rev ? alpha[0] : alpha[DEG];
      cd h = rev ? p[0] : p[DEG], hd = cd{0.0, 0.0};
#pragma unroll
      for (int k = 1; k <= DEG; ++k) {
        b = fma(b, ax, rev ? alpha[k] : alpha[DEG - k]);
        hd = add(mul(hd, x), h);
        h = add(mul(h, x), rev ? p[k] : p[DEG - k]);
      }
      if (absc(h) > __dmul_rn(EPS, b)) {
        cd s = cd{0.0, 0.0};
#pragma unroll
        for (int i = 0; i < DEG; ++i)
          if (i != j) s = add(s, recip(sub(z[j], z[i])));
        cd corr;
        if (rev) {
          cd z2h = mul(sq_pow(z[j]), h);
          corr = div(z2h, sub(sub(scale(mul(z[j], h), (double)DEG), hd), mul(z2h, s)));
        } else {
          corr = div(h, sub(hd, mul(h, s)));
        }
        z[j] = sub(z[j], corr);
      } else {
        conv |= 1u << j;
      }
    }
    if (conv == all) return it + 1;
  }
  return -1;
}

// The same iteration spread over a group of G lanes (DEG <= G <= 32; groups
// tile a warp from lane 0, so a warp holds 32 / G of them; every lane of the
// group calls it together): lane r owns root r.
// Root j's Horner values, stopping test and z_j^2 depend on z_j alone, which
// nothing changes before root j's own update, so all roots are evaluated at the
// start of an iteration; then, for j in order, the terms 1/(z_j - z_i) are formed on
// lanes i and summed in the serial order, and lane j applies its correction.
// The arithmetic of every value is that of solve(), so the iterates are the same
// bit for bit, at about a quarter of the sequential FP64 instructions.
// rank of this lane in its group, the group's first lane, and its lane mask
template <int G>
__device__ __forceinline__ int grank() {
  const int lane = threadIdx.x & 31;
  return ((G & (G - 1)) == 0) ? (lane & (G - 1)) : lane % G;
}
template <int G>
__device__ __forceinline__ unsigned gmask_of() {
  const int base = (threadIdx.x & 31) - grank<G>();
  return (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << base);
}
template <int G>
__device__ __forceinline__ cd gshfl(unsigned mask, cd v, int src) {
  if constexpr ((G & (G - 1)) == 0) {
    return cd{__shfl_sync(mask, v.x, src, G), __shfl_sync(mask, v.y, src, G)};
  } else {
    const int s = (threadIdx.x & 31) - grank<G>() + src;
    return cd{__shfl_sync(mask, v.x, s), __shfl_sync(mask, v.y, s)};
  }
}

// With `target` (the DEG converged roots of the same polynomial, from a fast
// solver) the iteration stops as soon as every iterate is clearly nearest one
// of them (nearest distance below half the second nearest) and no two iterates
// share a root: from there the iteration contracts each iterate onto that root,
// so the labelling it produces is already decided.
template <int DEG, int G>
__device__ int solve_group(const cd (&p)[DEG + 1], cd &zr, int itmax, bool warm, const cd *target = nullptr) {
  static_assert(G >= DEG && G <= 32, "group size");
  const int lane = threadIdx.x & 31, r = grank<G>();
  const unsigned gmask = gmask_of<G>();
  double alpha[DEG + 1];
#pragma unroll
  for (int i = 0; i <= DEG; ++i) alpha[i] = absc(p[i]);
  if (!warm) {
    cd t[DEG];
    init_real<DEG>(alpha, t);
    zr = cd{0.0, 0.0};
#pragma unroll
    for (int i = 0; i < DEG; ++i)
      if (i == r) zr = t[i];
  }
#pragma unroll
  for (int i = 0; i <= DEG; ++i) alpha[i] = __dmul_rn(alpha[i], fma(3.8284271247461900976, (double)i, 1.0));
  uint32_t conv = 0;
  const uint32_t all = (1u << DEG) - 1u;
  const double EPS = 1.1102230246251565e-16;
  for (int it = 0; it < itmax; ++it) {
    bool stop = false, rev = false;
    cd h = cd{0.0, 0.0}, hd = cd{0.0, 0.0}, zsq = cd{0.0, 0.0};
    if (r < DEG && !((conv >> r) & 1u)) {
      double az = absc(zr);
      rev = az > 1.0;
      cd x = rev ? recip(zr) : zr;
      double ax = rev ? __ddiv_rn(1.0, az) : az;
      double b = rev ? alpha[0] : alpha[DEG];
      h = rev ? p[0] : p[DEG];
#pragma unroll
      for (int k = 1; k <= DEG; ++k) {
        b = fma(b, ax, rev ? alpha[k] : alpha[DEG - k]);
        hd = add(mul(hd, x), h);
        h = add(mul(h, x), rev ? p[k] : p[DEG - k]);
      }
      stop = !(absc(h) > __dmul_rn(EPS, b));
      if (rev && !stop) zsq = sq_pow(zr);  // z_j^2 of the reversed correction, also from z_j alone
    }
    const uint32_t newly = (__ballot_sync(gmask, stop) >> (lane - r)) & all;
    for (int j = 0; j < DEG; ++j) {
      if (((conv | newly) >> j) & 1u) continue;  // uniform over the group
      const cd zj = gshfl<G>(gmask, zr, j);
      cd term = cd{0.0, 0.0};
      if (r < DEG && r != j) term = recip(sub(zj, zr));
      cd s = cd{0.0, 0.0};
#pragma unroll
      for (int i = 0; i < DEG; ++i) {
        const cd ti = gshfl<G>(gmask, term, i);
        if (i != j) s = add(s, ti);
      }
      if (r == j) {
        cd corr;
        if (rev) {
          cd z2h = mul(zsq, h);
          corr = div(z2h, sub(sub(scale(mul(zr, h), (double)DEG), hd), mul(z2h, s)));
        } else {
          corr = div(h, sub(hd, mul(h, s)));
        }
        zr = sub(zr, corr);
      }
    }
    conv |= newly;
    if (conv == all) return it + 1;
    if (target) {
      bool clear = true;
      uint32_t bit = 0;
      if (r < DEG) {
        double d1 = INFINITY, d2 = INFINITY;
        int best = 0;
#pragma unroll
        for (int j = 0; j < DEG; ++j) {
          const double d = norm2(target[j] - zr);
          if (d < d1) {
            d2 = d1;
            d1 = d;
            best = j;
          } else if (d < d2) {
            d2 = d;
          }
        }
        clear = d1 < 0.25 * d2;
        bit = 1u << best;
      }
      bit = __reduce_or_sync(gmask, bit);
      const bool all_clear = __all_sync(gmask, clear);
      if (all_clear && bit == all) return it + 1;
    }
  }
  return -1;
}

}  // namespace refea
