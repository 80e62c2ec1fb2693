// Ehrlich-Aberth simultaneous root solvers, one polynomial per thread, roots in
// registers (DEG is a compile-time constant so every array index is static).
//
// aberth64      FP64, the reference's iteration (lib/ehrlich_aberth/ehrlich_aberth.h:60-150):
//               Gauss-Seidel updates, reversed polynomial in 1/z when |z| > 1,
//               stop a root when |p(z)| <= EPS * sum |a_i| (1 + 3.828 i) |z|^i.
// aberth64_comp adds the reference's compensated second stage
//               (ehrlich_aberth.h:153-292) with an FP64 error-free Horner.
// aberth_mixed  FP32 iteration, then a compensated Horner stage in FP32 with
//               double-float coefficients (TwoSum / TwoProd via FMA) that drives
//               every root to float resolution against the FP64 polynomial, then
//               FP64 Newton polish; a root set that is not resolved falls back to
//               aberth64 from the polished roots.
//
// Initial estimates follow init_est.h:37-102 (radii from the upper convex hull
// of (i, log|a_i|)) but are complex: r*exp(i*phi).  The reference's guesses are
// real, r*sin(phi) (init_est.h:95), which only converge for real-coefficient
// polynomials through the rounding of thrust::pow.
#pragma once
#include "cplx.cuh"

#define CGB_EPS64 1.1102230246251565e-16
#define CGB_EPS32 5.9604644775390625e-08f

// per-item status bits (also exported in include/caustics_gb300.h)
#define CGB_ST_NOCONV 1u     // root solver reached itmax
#define CGB_ST_AMBIGUOUS 2u  // a lens-equation residual within x30 of the 1e-6 image threshold
#define CGB_ST_FALLBACK 4u   // mixed solver fell back to FP64 Aberth
#define CGB_ST_MERGE 8u      // contour linking left open segments or overflowed its buffer
#define CGB_ST_CAPACITY 16u  // limb / contour buffers too small for the request
#define CGB_ST_INVALID 32u   // a non-finite or out-of-domain input: the item's output is NaN

// real_guess: the reference's r*sin(phi) real initial guesses (init_est.h:95),
// used only to reproduce the reference's labelling of roots.
template <int DEG, typename R>
__device__ __forceinline__ void init_estimates(const R (&alpha)[DEG + 1], cd (&z)[DEG], bool real_guess = false) {
  double hx[DEG + 1], hy[DEG + 1], al[DEG + 1];
#pragma unroll
  for (int i = 0; i <= DEG; ++i) al[i] = (double)alpha[i];
  int k = 0;
  for (int i = DEG; i >= 0; --i) {
    double y = al[i] > 0 ? log(al[i]) : -1e30;
    while (k >= 2 && (hx[k - 1] - hx[k - 2]) * (y - hy[k - 2]) - (hy[k - 1] - hy[k - 2]) * ((double)i - hx[k - 2]) <= 0)
      --k;
    hx[k] = i;
    hy[k] = y;
    ++k;
  }
  cd t[DEG];
  const double pi2 = 6.28318530717958647693, th = pi2 / DEG;
  int n = 0;
  for (int i = k - 2; i >= 0; --i) {
    int nz = (int)(hx[i] - hx[i + 1]);
    double r = real_guess ? pow(al[(int)hx[i + 1]], 1.0 / nz) / pow(al[(int)hx[i]], 1.0 / nz)
                          : exp((hy[i + 1] - hy[i]) / nz);
    if (!(r > 0.0) || !isfinite(r)) r = 1.0;
    double ang = pi2 / nz;
    for (int j = 0; j < nz && n + j < DEG; ++j) {
      double s, c;
      sincos(ang * j + th * i + 0.7, &s, &c);
      t[n + j] = real_guess ? mk(r * s, 0.0) : mk(r * c, r * s);
    }
    n += nz;
  }
#pragma unroll
  for (int i = 0; i < DEG; ++i) z[i] = t[i];
}

// The same initial estimates in FP32 arithmetic, for the mixed solver whose
// FP32 iteration starts from them (the FP64 transcendentals would cost several
// hundred FP64 instructions per polynomial on a part with a narrow FP64 pipe).
template <int DEG>
__device__ __forceinline__ void init_estimates_f32(const float (&alpha)[DEG + 1], cf (&z)[DEG]) {
  int hx[DEG + 1];
  float hy[DEG + 1];
  int k = 0;
  for (int i = DEG; i >= 0; --i) {
    const float y = alpha[i] > 0.0f ? logf(alpha[i]) : -1e30f;
    while (k >= 2 &&
           (float)(hx[k - 1] - hx[k - 2]) * (y - hy[k - 2]) - (hy[k - 1] - hy[k - 2]) * (float)(i - hx[k - 2]) <= 0.0f)
      --k;
    hx[k] = i;
    hy[k] = y;
    ++k;
  }
  cf t[DEG];
  const float pi2 = 6.28318530717958647693f, th = pi2 / DEG;
  int n = 0;
  for (int i = k - 2; i >= 0; --i) {
    const int nz = hx[i] - hx[i + 1];
    float r = expf((hy[i + 1] - hy[i]) / (float)nz);
    if (!(r > 0.0f) || !isfinite(r)) r = 1.0f;
    const float ang = pi2 / (float)nz;
    for (int j = 0; j < nz && n + j < DEG; ++j) {
      float sn, cs;
      sincosf(ang * (float)j + th * (float)i + 0.7f, &sn, &cs);
      t[n + j] = mkf(r * cs, r * sn);
    }
    n += nz;
  }
#pragma unroll
  for (int i = 0; i < DEG; ++i) z[i] = t[i];
}

// sum_{i != j} 1 / (z_j - z_i)
template <int DEG, typename C>
__device__ __forceinline__ C aberth_sum(const C (&z)[DEG], int j) {
  C s = z[0] - z[0];
#pragma unroll
  for (int i = 0; i < DEG; ++i)
    if (i != j) s = s + crecip(z[j] - z[i]);
  return s;
}

// Horner for p and p' at x; rev walks the coefficients from p[0] (the reversed
// polynomial evaluated at x = 1/z).  b = the real bound polynomial at |x|.
template <int DEG, typename C, typename R>
__device__ __forceinline__ void horner_pair(const C (&p)[DEG + 1], const R (&alpha)[DEG + 1], C x, R ax, bool rev,
                                            C &h, C &hd, R &b) {
  h = rev ? p[0] : p[DEG];
  b = rev ? alpha[0] : alpha[DEG];
  hd = h - h;
#pragma unroll
  for (int k = 1; k <= DEG; ++k) {
    C pk = rev ? p[k] : p[DEG - k];
    R ak = rev ? alpha[k] : alpha[DEG - k];
    hd = cfma(hd, x, h);
    h = cfma(h, x, pk);
    b = b * ax + ak;
  }
}

// Aberth correction; rev form from ehrlich_aberth.h:43-58
__device__ __forceinline__ cd sq_powform(cd z) {
  // z^2 as thrust::pow(z, 2) = exp(2 log z) forms it (ehrlich_aberth.h:56-57)
  double m = exp(2.0 * log(sqrt(z.x * z.x + z.y * z.y))), t = 2.0 * atan2(z.y, z.x), s, c;
  sincos(t, &s, &c);
  return mk(m * c, m * s);
}
__device__ __forceinline__ cf sq_powform(cf z) { return z * z; }

template <int DEG, typename C, bool POWSQ = false>
__device__ __forceinline__ C aberth_corr(const C (&z)[DEG], int j, C h, C hd, bool rev) {
  C s = aberth_sum<DEG, C>(z, j);
  if (rev) {
    C z2h = (POWSQ ? sq_powform(z[j]) : z[j] * z[j]) * h;
    C d = z[j] * h;
    d = C{d.x * DEG, d.y * DEG} - hd - z2h * s;
    return cdiv(z2h, d);
  }
  return cdiv(h, hd - h * s);
}

// REF: the reference's real initial guesses and pow-form square, to reproduce
// its labelling of roots (row order) on a cold start.
template <int DEG, bool REF = false>
__device__ int aberth64(const cd (&p)[DEG + 1], cd (&z)[DEG], int itmax, bool warm) {
  double alpha[DEG + 1];
#pragma unroll
  for (int i = 0; i <= DEG; ++i) alpha[i] = cabs(p[i]);
  if (!warm) init_estimates<DEG>(alpha, z, REF);
#pragma unroll
  for (int i = 0; i <= DEG; ++i) alpha[i] *= fma(3.8284271247461900976, (double)i, 1.0);
  uint32_t conv = 0;
  const uint32_t all = (1u << DEG) - 1u;
  for (int it = 0; it < itmax; ++it) {
#pragma unroll
    for (int j = 0; j < DEG; ++j) {
      if (!((conv >> j) & 1u)) {
        double az = cabs(z[j]);
        bool rev = az > 1.0;
        cd x = rev ? crecip(z[j]) : z[j];
        cd h, hd;
        double b;
        horner_pair<DEG>(p, alpha, x, rev ? 1.0 / az : az, rev, h, hd, b);
        if (cabs(h) > CGB_EPS64 * b)
          z[j] = z[j] - aberth_corr<DEG, cd, REF>(z, j, h, hd, rev);
        else
          conv |= 1u << j;
      }
    }
    if (conv == all) return it + 1;
  }
  return -1;
}

// Compensated Horner (error-free transforms) for p and p' at x, optionally with
// a low-order coefficient part pl (double-float coefficients).  Returns the
// compensated h, hd and the running error bound eb (horner.h:281-385).
template <int DEG, typename C, typename R>
__device__ __forceinline__ void horner_comp(const C (&p)[DEG + 1], const C (&pl)[DEG + 1], bool use_lo, C x,
                                            bool rev, C &h_out, C &hd_out, R &eb) {
  C H = rev ? p[0] : p[DEG];
  C e = use_lo ? (rev ? pl[0] : pl[DEG]) : H - H;
  C D = H - H, ed = H - H;
  R ax = msqrt(x.x * x.x + x.y * x.y);
  eb = 0;
#pragma unroll
  for (int k = 1; k <= DEG; ++k) {
    C pk = rev ? p[k] : p[DEG - k];
    // D*x + H
    R p0, q0, p1, q1, p2, q2, p3, q3, s4, r4, s5, r5, sx, ex, sy, ey;
    two_prod(D.x, x.x, p0, q0);
    two_prod(D.y, x.y, p1, q1);
    two_prod(D.x, x.y, p2, q2);
    two_prod(D.y, x.x, p3, q3);
    two_sum(p0, -p1, s4, r4);
    two_sum(p2, p3, s5, r5);
    two_sum(s4, H.x, sx, ex);
    two_sum(s5, H.y, sy, ey);
    D = C{sx, sy};
    ed = cfma(ed, x, e) + C{(q0 - q1) + (r4 + ex), (q2 + q3) + (r5 + ey)};
    // H*x + p_k
    two_prod(H.x, x.x, p0, q0);
    two_prod(H.y, x.y, p1, q1);
    two_prod(H.x, x.y, p2, q2);
    two_prod(H.y, x.x, p3, q3);
    two_sum(p0, -p1, s4, r4);
    two_sum(p2, p3, s5, r5);
    two_sum(s4, pk.x, sx, ex);
    two_sum(s5, pk.y, sy, ey);
    H = C{sx, sy};
    C lo = C{(q0 - q1) + (r4 + ex), (q2 + q3) + (r5 + ey)};
    if (use_lo) lo = lo + (rev ? pl[k] : pl[DEG - k]);
    e = cfma(e, x, lo);
    eb = eb * ax + (mabs(q0) + mabs(q1) + mabs(q2) + mabs(q3) + mabs(r4) + mabs(r5) + mabs(ex) + mabs(ey));
  }
  h_out = H + e;
  hd_out = D + ed;
}

template <typename R>
__device__ __forceinline__ R gamma_const(unsigned n, R eps) {
  R g = (R)(2 * n) * eps * (R)1.41421356237309504880;
  return g / (((R)1 - (R)2 * eps) - g);
}

// The reference's compensated solver: stage 1 as aberth64, stage 2 with the
// compensated error bound (ehrlich_aberth.h:229-273).
template <int DEG>
__device__ int aberth64_comp(const cd (&p)[DEG + 1], cd (&z)[DEG], int itmax, bool warm) {
  double alpha[DEG + 1];
#pragma unroll
  for (int i = 0; i <= DEG; ++i) alpha[i] = cabs(p[i]);
  if (!warm) init_estimates<DEG>(alpha, z);
#pragma unroll
  for (int i = 0; i <= DEG; ++i) alpha[i] *= fma(3.8284271247461900976, (double)i, 1.0);
  uint32_t cx = 0, cy = 0;
  const uint32_t all = (1u << DEG) - 1u;
  const double gam = gamma_const<double>(4 * DEG + 2, CGB_EPS64);
  for (int it = 0; it < itmax; ++it) {
#pragma unroll
    for (int j = 0; j < DEG; ++j) {
      double az = cabs(z[j]);
      bool rev = az > 1.0;
      cd x = rev ? crecip(z[j]) : z[j];
      if (!((cx >> j) & 1u)) {
        cd h, hd;
        double b;
        horner_pair<DEG>(p, alpha, x, rev ? 1.0 / az : az, rev, h, hd, b);
        if (cabs(h) > CGB_EPS64 * b)
          z[j] = z[j] - aberth_corr<DEG>(z, j, h, hd, rev);
        else
          cx |= 1u << j;
      } else if (!((cy >> j) & 1u)) {
        cd h, hd;
        double eb;
        horner_comp<DEG, cd, double>(p, p, false, x, rev, h, hd, eb);
        double ah = cabs(h);
        double bound = CGB_EPS64 * ah + (gam * eb + 2 * CGB_EPS64 * CGB_EPS64 * ah);
        if (ah > 4 * bound) {
          cd c = aberth_corr<DEG>(z, j, h, hd, rev);
          double lim = rev ? 4 * CGB_EPS64 * az : 4 * CGB_EPS64;
          if (cabs(c) > lim)
            z[j] = z[j] - c;
          else
            cy |= 1u << j;
        } else {
          cy |= 1u << j;
        }
      }
    }
    if (cy == all) return it + 1;
  }
  return -1;
}

// No two roots closer than 1e-7 of the largest root's modulus.  A root set
// that fails this is not trusted (two starts may have converged onto one root,
// leaving another root unfound).
template <int DEG>
__device__ __forceinline__ bool roots_distinct(const cd (&z)[DEG]) {
  double scale = 0.0;
#pragma unroll
  for (int i = 0; i < DEG; ++i) scale = fmax(scale, norm2(z[i]));
  bool ok = true;
#pragma unroll
  for (int i = 0; i < DEG; ++i)
#pragma unroll
    for (int k = i + 1; k < DEG; ++k)
      if (norm2(z[i] - z[k]) < 1e-14 * scale) ok = false;
  return ok;
}

// FP64 fallback of the mixed solver.  It never warm-starts from a set with
// merged roots: with two coincident starts the Aberth correction of the pair
// degenerates and both can settle on one root.  warm (if given) is a start known
// to separate the roots (e.g. the neighbouring limb point's roots plus jitter);
// otherwise, or if that fails or merges roots, a cold start.  Returns the FP64
// iteration count or -1.  Not inlined: it runs rarely, and its body would
// otherwise enter the register allocation of every kernel that can fall back.
template <int DEG>
__device__ __noinline__ int aberth64_fallback(const cd (&p)[DEG + 1], cd (&z)[DEG], int itmax, const cd *warm) {
  int it = -1;
  if (warm) {  // a warm start converges in a few iterations or not at all
#pragma unroll
    for (int i = 0; i < DEG; ++i) z[i] = warm[i];
    it = aberth64<DEG>(p, z, min(itmax, 64), true);
    if (it >= 0 && roots_distinct<DEG>(z)) return it;
  }
  it = aberth64<DEG>(p, z, itmax, false);
  return (it >= 0 && roots_distinct<DEG>(z)) ? it : -1;
}

// The mixed solver's FP64 fallback from the roots it found: each moved by
// 1e-6 in its own direction, which separates a pair Newton merged, so the FP64
// iteration needs a few steps where a cold start needs tens; cold if that
// fails.  Not inlined, like aberth64_fallback.
template <int DEG>
__device__ __noinline__ int aberth64_fallback_separated(const cd (&p)[DEG + 1], cd (&z)[DEG], int itmax) {
  cd start[DEG];
  bool finite = true;
#pragma unroll
  for (int i = 0; i < DEG; ++i) {
    double sn, cs;
    sincospi(2.0 * i / DEG, &sn, &cs);
    start[i] = z[i] + mk(1e-6 * cs, 1e-6 * sn);
    finite = finite && isfinite(start[i].x) && isfinite(start[i].y);
  }
  return aberth64_fallback<DEG>(p, z, itmax, finite ? start : nullptr);
}

// FP64 Aberth iteration spread over a group of G lanes (G a power of two, DEG
// <= G <= 32; every lane of the group calls it, gmask its lanes): lane r < DEG
// owns root r (zr, from a start that separates the roots) and all roots update
// together from the previous iterate; each root stops at the reference's FP64
// rule.  Returns, uniformly over the group, whether every root stopped within
// itmax iterations with finite values.
template <int DEG, int G>
__device__ bool aberth64_group(const cd (&p)[DEG + 1], cd &zr, int itmax, unsigned gmask) {
  const int r = threadIdx.x & (G - 1);
  double alpha[DEG + 1];
#pragma unroll
  for (int i = 0; i <= DEG; ++i) alpha[i] = cabs(p[i]) * fma(3.8284271247461900976, (double)i, 1.0);
  bool done = r >= DEG;
  for (int it = 0; it < itmax; ++it) {
    cd zall[DEG];
#pragma unroll
    for (int q = 0; q < DEG; ++q) zall[q] = mk(__shfl_sync(gmask, zr.x, q, G), __shfl_sync(gmask, zr.y, q, G));
    if (!done) {
      const double az = cabs(zr);
      const bool rev = az > 1.0;
      const cd x = rev ? crecip(zr) : zr;
      cd h, hd;
      double b;
      horner_pair<DEG>(p, alpha, x, rev ? 1.0 / az : az, rev, h, hd, b);
      if (cabs(h) > CGB_EPS64 * b) {
        cd sum = mk(0.0, 0.0);
#pragma unroll
        for (int q = 0; q < DEG; ++q)
          if (q != r) sum = sum + crecip(zr - zall[q]);
        cd corr;
        if (rev) {
          const cd z2h = (zr * zr) * h, d = zr * h;
          corr = cdiv(z2h, mk(d.x * DEG, d.y * DEG) - hd - z2h * sum);
        } else {
          corr = cdiv(h, hd - h * sum);
        }
        zr = zr - corr;
      } else {
        done = true;
      }
    }
    if (__all_sync(gmask, done)) return __all_sync(gmask, isfinite(zr.x) && isfinite(zr.y));
  }
  return false;
}

// The FP32 Aberth stage on a group of G lanes, lane r < DEG iterating root r
// from zr (every root updated from the previous iterate, roots exchanged by
// shuffles), with the FP32 stopping rule of the reference's iteration; alpha =
// |p_i| (1 + 3.8284271247461900976 i).  True when every root met the rule
// within itcap iterations with finite values.
template <int DEG, int G>
__device__ bool aberth32_group(const cf (&ph)[DEG + 1], const float (&alpha)[DEG + 1], cf &zr, unsigned gmask,
                               int itcap) {
  const int r = threadIdx.x & (G - 1);
  bool done = r >= DEG;
  for (int it = 0; it < itcap; ++it) {
    cf zall[DEG];
#pragma unroll
    for (int q = 0; q < DEG; ++q) zall[q] = mkf(__shfl_sync(gmask, zr.x, q, G), __shfl_sync(gmask, zr.y, q, G));
    if (!done) {
      const float az = cabs(zr);
      const bool rev = az > 1.0f;
      const cf x = rev ? crecip(zr) : zr;
      cf h, hd;
      float b;
      horner_pair<DEG>(ph, alpha, x, rev ? 1.0f / az : az, rev, h, hd, b);
      if (cabs(h) > CGB_EPS32 * b) {
        cf sum = mkf(0.0f, 0.0f);
#pragma unroll
        for (int q = 0; q < DEG; ++q)
          if (q != r) sum = sum + crecip(zr - zall[q]);
        cf corr;
        if (rev) {
          const cf z2h = (zr * zr) * h, d = zr * h;
          corr = cdiv(z2h, mkf(d.x * DEG, d.y * DEG) - hd - z2h * sum);
        } else {
          corr = cdiv(h, hd - h * sum);
        }
        zr = zr - corr;
      } else {
        done = true;
      }
    }
    if (__all_sync(gmask, done)) return __all_sync(gmask, isfinite(zr.x) && isfinite(zr.y));
  }
  return false;
}

// FP64 Newton on one root of p (low -> high): at most SWEEPS steps, done when a
// correction is at most 2^-40 |z|.  With sep2 = S^2 (default: infinite, the
// plain rule only), S = sum_{k != j} 1/|z - z_k|
// over the other roots, a step is also final when Newton's error model puts
// the next correction, |c|^2 |p''/(2p')| = |c|^2 |sum_k 1/(z - z_k)| <= |c|^2 S,
// at most 2^-40 |z|: from an FP32 root (relative error ~1e-7) one step then
// leaves ~1e-13, where the plain rule needs a second step to see it.
template <int DEG, int SWEEPS = 3>
__device__ bool newton_polish_root(const cd (&p)[DEG + 1], cd &z, float sep2 = INFINITY) {
  for (int sweep = 0; sweep < SWEEPS; ++sweep) {
    cd h = p[DEG], hd = mk(0, 0);
#pragma unroll
    for (int k = DEG - 1; k >= 0; --k) {
      hd = cfma(hd, z, h);
      h = cfma(h, z, p[k]);
    }
    const cd c = cdiv(h, hd);
    z = z - c;
    const double c2 = norm2(c), z2 = 8.271806125530277e-25 * fmax(norm2(z), 1e-300);
    if (c2 <= z2 || c2 * c2 * (double)sep2 <= z2) return true;
  }
  return false;
}

// S_j^2, S_j = sum_{k != j} 1/|z_j - z_k| (FP32), for newton_polish_root's
// error model; infinite for coincident roots, which then never stop early.
template <int DEG>
__device__ __forceinline__ void root_separation2(const cf (&z)[DEG], float (&s2)[DEG]) {
#pragma unroll
  for (int j = 0; j < DEG; ++j) {
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < DEG; ++k)
      if (k != j) s += rsqrtf(norm2(z[j] - z[k]));
    s2[j] = s * s;
  }
}

// Mixed precision: FP32 Aberth, FP32 compensated stage against the double-float
// polynomial, FP64 Newton polish, FP64 fallback.  Returns the FP32 iteration
// count, -1 on non-convergence; sets CGB_ST_FALLBACK in flags when used.
// WARM_FALLBACK: the FP64 fallback first starts from the roots found so far,
// each moved by 1e-6 in its own direction (that separates a pair Newton merged;
// a few FP64 steps then replace the tens of a cold start).  It suits the
// one-polynomial-per-thread kernels, where a warp waits for its slowest lane;
// in the contour kernel it measured slower (the chained matching that follows
// ran 50 % longer with that code present), so that kernel starts cold.
// EARLY: each root's polish may stop after one step on newton_polish_root's
// error model (roots to ~1e-13 instead of ~1e-16; the contour kernel's limb
// solves, whose results need 1e-4); the point-source kernels keep the plain rule.
template <int DEG, bool WARM_FALLBACK = false, bool EARLY = false>
__device__ int aberth_mixed(const cd (&p)[DEG + 1], cd (&z)[DEG], int itmax, bool warm, uint32_t &flags) {
  cf ph[DEG + 1], pl[DEG + 1];
  float alpha[DEG + 1];
#pragma unroll
  for (int i = 0; i <= DEG; ++i) {
    ph[i] = tof(p[i]);
    pl[i] = tof(p[i] - tod(ph[i]));
    alpha[i] = cabs(ph[i]);
  }
  cf zf[DEG];
  if (warm) {
#pragma unroll
    for (int i = 0; i < DEG; ++i) zf[i] = tof(z[i]);
  } else {
    init_estimates_f32<DEG>(alpha, zf);
  }
#pragma unroll
  for (int i = 0; i <= DEG; ++i) alpha[i] *= fmaf(3.8284271247461900976f, (float)i, 1.0f);
  const float gam = gamma_const<float>(4 * DEG + 2, CGB_EPS32);
  uint32_t cx = 0, cy = 0;
  const uint32_t all = (1u << DEG) - 1u;
  // Two loops rather than the reference's one (where a root starts its
  // compensated steps while others still run plain ones): a warp runs the
  // costly compensated evaluation only while one of its lanes needs it, and
  // lanes reach that stage at different iterations.  The FP32 stopping rule
  // sits at FP32's own Horner rounding level, so a converged root can keep
  // missing it: the FP32 stage stops after 128 iterations and such roots go on
  // to the compensated stage (at most 64 iterations), whose double-float
  // evaluation can meet its bound.  Whatever still fails takes the FP64
  // fallback below.
  int it = 0;
  const int it32 = min(itmax, 128);
  for (; it < it32 && cx != all; ++it) {
#pragma unroll
    for (int j = 0; j < DEG; ++j) {
      if ((cx >> j) & 1u) continue;
      const float az = cabs(zf[j]);
      const bool rev = az > 1.0f;
      const cf x = rev ? crecip(zf[j]) : zf[j];
      cf h, hd;
      float b;
      horner_pair<DEG>(ph, alpha, x, rev ? 1.0f / az : az, rev, h, hd, b);
      if (cabs(h) > CGB_EPS32 * b)
        zf[j] = zf[j] - aberth_corr<DEG>(zf, j, h, hd, rev);
      else
        cx |= 1u << j;
    }
  }
  const int itc = min(itmax, it + 64);
  for (; it < itc && cy != all; ++it) {
#pragma unroll
    for (int j = 0; j < DEG; ++j) {
      if ((cy >> j) & 1u) continue;
      const float az = cabs(zf[j]);
      const bool rev = az > 1.0f;
      const cf x = rev ? crecip(zf[j]) : zf[j];
      cf h, hd;
      float eb;
      horner_comp<DEG, cf, float>(ph, pl, true, x, rev, h, hd, eb);
      const float ah = cabs(h);
      const float bound = CGB_EPS32 * ah + (gam * eb + 2 * CGB_EPS32 * CGB_EPS32 * ah);
      if (ah > 4 * bound) {
        const cf c = aberth_corr<DEG>(zf, j, h, hd, rev);
        if (cabs(c) > 4 * CGB_EPS32 * az)
          zf[j] = zf[j] - c;
        else
          cy |= 1u << j;
      } else {
        cy |= 1u << j;
      }
    }
  }
  bool ok = (cy == all) && isfinite(zf[0].x);
#pragma unroll
  for (int i = 0; i < DEG; ++i) z[i] = tod(zf[i]);
  // FP64 Newton polish (forward Horner; degrees are small), done when every
  // correction is at most 2^-40 |z| (compared without a division; a NaN
  // correction never passes)
  bool conv = false;
  if constexpr (EARLY) {
    float s2[DEG];
    root_separation2<DEG>(zf, s2);
    uint32_t done = 0;
    for (int sweep = 0; sweep < 3 && ok && done != all; ++sweep) {
#pragma unroll
      for (int j = 0; j < DEG; ++j) {
        if ((done >> j) & 1u) continue;
        cd h = p[DEG], hd = mk(0, 0);
#pragma unroll
        for (int k = DEG - 1; k >= 0; --k) {
          hd = cfma(hd, z[j], h);
          h = cfma(h, z[j], p[k]);
        }
        const cd c = cdiv(h, hd);
        z[j] = z[j] - c;
        const double c2 = norm2(c), z2 = 8.271806125530277e-25 * fmax(norm2(z[j]), 1e-300);
        if (c2 <= z2 || c2 * c2 * (double)s2[j] <= z2) done |= 1u << j;
      }
    }
    conv = done == all;
  } else {
    for (int sweep = 0; sweep < 3 && ok; ++sweep) {
      conv = true;
#pragma unroll
      for (int j = 0; j < DEG; ++j) {
        cd h = p[DEG], hd = mk(0, 0);
#pragma unroll
        for (int k = DEG - 1; k >= 0; --k) {
          hd = cfma(hd, z[j], h);
          h = cfma(h, z[j], p[k]);
        }
        cd c = cdiv(h, hd);
        z[j] = z[j] - c;
        conv = conv && norm2(c) <= 8.271806125530277e-25 * fmax(norm2(z[j]), 1e-300);
      }
      if (conv) break;
    }
  }
  ok = ok && conv;
  // distinct roots (Newton alone may merge a near-double pair)
  if (ok) {
    double scale = 0.0;
#pragma unroll
    for (int i = 0; i < DEG; ++i) scale = fmax(scale, norm2(z[i]));
#pragma unroll
    for (int i = 0; i < DEG; ++i)
#pragma unroll
      for (int k = i + 1; k < DEG; ++k)
        if (norm2(z[i] - z[k]) < 1e-14 * scale) ok = false;
  }
  if (!ok) {
    flags |= CGB_ST_FALLBACK;
    if constexpr (WARM_FALLBACK) {
      if (aberth64_fallback_separated<DEG>(p, z, itmax) < 0) return -1;
    } else {
      if (aberth64_fallback<DEG>(p, z, itmax, nullptr) < 0) return -1;
    }
  }
  return it + 1;
}
