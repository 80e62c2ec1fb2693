// Point-source kernels: the Ehrlich-Aberth solver as a batched primitive
// (replaces the XLA custom call of lib/ehrlich_aberth/kernels.cc.cu:14-42),
// fused point-source magnification (src/caustics/point_source.py:1652-1830), and
// the per-point pass of the light-curve driver (src/caustics/lightcurve.py:99-227).
//
// One polynomial per thread with roots and coefficients in registers.  Global
// traffic is staged through shared memory so that every warp moves contiguous
// 16-byte words (coefficients in, roots out).
//
// The solver precision is a template parameter: each kernel holds one solver,
// so its register allocation (and with it the occupancy) is that solver's own,
// not the largest of the three.  ps_fp64.cu, ps_mixed.cu and ps_comp.cu each
// instantiate one precision; point_source.cu dispatches on the runtime value.
#pragma once
#include "aberth.cuh"
#include "hexadecapole.cuh"
#include "es.h"
#include "internal.h"

namespace cgb {

constexpr int PS_THREADS = 128;

template <int PREC, int DEG>
__device__ __forceinline__ int solve(const cd (&p)[DEG + 1], cd (&z)[DEG], int itmax, bool warm, uint32_t &flags) {
  if constexpr (PREC == MIXED) return aberth_mixed<DEG, true>(p, z, itmax, warm, flags);
  else if constexpr (PREC == FP64_COMP) return aberth64_comp<DEG>(p, z, itmax, warm);
  else return aberth64<DEG>(p, z, itmax, warm);
}

// coeffs: complex128 [n, DEG+1] low->high; roots_init: complex128 [n, DEG] or null.
template <int PREC, int DEG>
__global__ void __launch_bounds__(PS_THREADS) ea_solve_kernel(const cd *__restrict__ coeffs,
                                                              const cd *__restrict__ roots_init,
                                                              cd *__restrict__ roots, int64_t n, int itmax,
                                                              uint32_t *__restrict__ status) {
  __shared__ cd stage[PS_THREADS * (DEG + 1)];
  const int64_t base = (int64_t)blockIdx.x * PS_THREADS;
  const int tid = threadIdx.x;
  const int64_t cnt = min((int64_t)PS_THREADS, n - base);
  // coalesced load of this block's coefficients
  for (int i = tid; i < cnt * (DEG + 1); i += PS_THREADS) stage[i] = coeffs[base * (DEG + 1) + i];
  __syncthreads();
  cd p[DEG + 1], z[DEG];
  bool active = tid < cnt;
  if (active) {
#pragma unroll
    for (int k = 0; k <= DEG; ++k) p[k] = stage[tid * (DEG + 1) + k];
  }
  __syncthreads();
  if (roots_init) {
    for (int i = tid; i < cnt * DEG; i += PS_THREADS) stage[i] = roots_init[base * DEG + i];
    __syncthreads();
    if (active) {
#pragma unroll
      for (int k = 0; k < DEG; ++k) z[k] = stage[tid * DEG + k];
    }
    __syncthreads();
  }
  uint32_t flags = 0;
  if (active) {
    bool finite = true;
#pragma unroll
    for (int k = 0; k <= DEG; ++k) finite &= isfinite(p[k].x) && isfinite(p[k].y);
    if (finite) {
      int it = solve<PREC, DEG>(p, z, itmax, roots_init != nullptr, flags);
      if (it < 0) flags |= CGB_ST_NOCONV;
    } else {  // not solved: NaN roots
      flags = CGB_ST_INVALID;
      const double nan = __longlong_as_double(0x7ff8000000000000ll);
#pragma unroll
      for (int k = 0; k < DEG; ++k) z[k] = mk(nan, nan);
    }
#pragma unroll
    for (int k = 0; k < DEG; ++k) stage[tid * DEG + k] = z[k];
    if (status) status[base + tid] = flags;
  }
  __syncthreads();
  for (int i = tid; i < cnt * DEG; i += PS_THREADS) roots[base * DEG + i] = stage[i];
}

template <int PREC>
cudaError_t launch_ea_solve_p(const double *coeffs, const double *roots_init, double *roots, int64_t n, int deg,
                              int itmax, uint32_t *status, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  dim3 grid((unsigned)((n + PS_THREADS - 1) / PS_THREADS));
  const cd *c = reinterpret_cast<const cd *>(coeffs);
  const cd *ri = reinterpret_cast<const cd *>(roots_init);
  cd *r = reinterpret_cast<cd *>(roots);
  switch (deg) {
    case 4: ea_solve_kernel<PREC, 4><<<grid, PS_THREADS, 0, stream>>>(c, ri, r, n, itmax, status); break;
    case 5: ea_solve_kernel<PREC, 5><<<grid, PS_THREADS, 0, stream>>>(c, ri, r, n, itmax, status); break;
    case 6: ea_solve_kernel<PREC, 6><<<grid, PS_THREADS, 0, stream>>>(c, ri, r, n, itmax, status); break;
    case 10: ea_solve_kernel<PREC, 10><<<grid, PS_THREADS, 0, stream>>>(c, ri, r, n, itmax, status); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// Images of one (shifted) source position; returns the real-image bit mask and
// raises CGB_ST_AMBIGUOUS when a residual sits within x30 of the 1e-6 threshold.
template <int PREC, int NL>
__device__ __forceinline__ uint32_t images(const Lens &L, cd w, cd (&z)[NL * NL + 1], int itmax, uint32_t &flags) {
  constexpr int DEG = NL * NL + 1;
  cd p[DEG + 1];
  lens_poly<NL>(L, w, p);
  int it = solve<PREC, DEG>(p, z, itmax, false, flags);
  if (it < 0) flags |= CGB_ST_NOCONV;
  uint32_t mask = 0;
#pragma unroll
  for (int i = 0; i < DEG; ++i) {
    double r = cabs(lens_eq<NL>(L, z[i]) - w);
    if (r < 1e-6) mask |= 1u << i;
    if (r > 1e-6 / 30 && r < 1e-6 * 30) flags |= CGB_ST_AMBIGUOUS;
  }
  return mask;
}

// images() on a group of G lanes (binary lenses): lane r < DEG iterates root
// r of the point's polynomial, all roots updated together and exchanged by
// shuffles, from FP32 initial estimates.  Mixed precision: the FP32 stage,
// then an FP64 Newton polish of each lane's root and a distinctness check,
// with the FP64 group iteration as the fallback; FP64: the FP64 group
// iteration.  Every lane of the group calls it and gets all roots and the mask.
template <int PREC, int G>
__device__ uint32_t images_group(const Lens &L, cd w, cd (&z)[5], int itmax, uint32_t &flags, unsigned gmask) {
  constexpr int DEG = 5;
  const int r = threadIdx.x & (G - 1), gbase = (threadIdx.x & 31) - r;
  cd p[DEG + 1];
  lens_poly<2>(L, w, p);
  cf ph[DEG + 1];
  float alpha[DEG + 1];
#pragma unroll
  for (int i = 0; i <= DEG; ++i) {
    ph[i] = tof(p[i]);
    alpha[i] = cabs(ph[i]);
  }
  cf z0[DEG];
  init_estimates_f32<DEG>(alpha, z0);
  cf zf = z0[0];
#pragma unroll
  for (int q = 1; q < DEG; ++q)
    if (q == r) zf = z0[q];
  const cf zstart = zf;
#pragma unroll
  for (int i = 0; i <= DEG; ++i) alpha[i] *= fmaf(3.8284271247461900976f, (float)i, 1.0f);
  cd zr;
  bool ok;
  if constexpr (PREC == MIXED) {
    ok = aberth32_group<DEG, G>(ph, alpha, zf, gmask, min(itmax, 128));
    zr = tod(zf);
    const bool conv = r >= DEG || newton_polish_root<DEG, 5>(p, zr);
    ok = __all_sync(gmask, ok && conv);
    if (ok) {  // distinct roots (Newton alone may merge a near-double pair)
      double scale = 0.0;
      bool sep = true;
#pragma unroll
      for (int q = 0; q < DEG; ++q) {
        const cd zq = mk(__shfl_sync(gmask, zr.x, q, G), __shfl_sync(gmask, zr.y, q, G));
        scale = fmax(scale, norm2(zq));
        if (r < DEG && q > r && norm2(zr - zq) < 1e-14 * fmax(norm2(zr), norm2(zq))) sep = false;
      }
      ok = __all_sync(gmask, sep);
    }
    if (!ok) {
      flags |= CGB_ST_FALLBACK;
      zr = tod(zstart);
      ok = aberth64_group<DEG, G>(p, zr, itmax, gmask);
    }
  } else {
    zr = tod(zstart);
    ok = aberth64_group<DEG, G>(p, zr, itmax, gmask);
  }
  if (!ok) flags |= CGB_ST_NOCONV;
#pragma unroll
  for (int q = 0; q < DEG; ++q) z[q] = mk(__shfl_sync(gmask, zr.x, q, G), __shfl_sync(gmask, zr.y, q, G));
  const double res = r < DEG ? cabs(lens_eq<2>(L, zr) - w) : 1.0;
  const uint32_t mask = (__ballot_sync(gmask, r < DEG && res < 1e-6) >> gbase) & ((1u << DEG) - 1u);
  if (__any_sync(gmask, r < DEG && res > 1e-6 / 30 && res < 1e-6 * 30)) flags |= CGB_ST_AMBIGUOUS;
  return mask;
}

template <int PREC, int NL>
__global__ void __launch_bounds__(PS_THREADS) mag_ps_kernel(Lens L, const cd *__restrict__ w, double *__restrict__ mag,
                                                            cd *__restrict__ images_out,
                                                            uint32_t *__restrict__ mask_out, int64_t n, int itmax,
                                                            uint32_t *__restrict__ status) {
  constexpr int DEG = NL * NL + 1;
  __shared__ cd stage[PS_THREADS * DEG];
  const int64_t base = (int64_t)blockIdx.x * PS_THREADS;
  const int tid = threadIdx.x;
  const int64_t i = base + tid;
  const int64_t cnt = min((int64_t)PS_THREADS, n - base);
  cd z[DEG];
  uint32_t flags = 0, m = 0;
  if (i < n) {
    cd wi = w[i];
    double mu = 0.0;
    if (isfinite(wi.x) && isfinite(wi.y)) {
      wi.x += L.x_cm;
      m = images<PREC, NL>(L, wi, z, itmax, flags);
#pragma unroll
      for (int k = 0; k < DEG; ++k)
        if ((m >> k) & 1u) mu += 1.0 / fabs(lens_det<NL>(L, z[k]));
    } else {  // not solved: NaN magnification and images
      flags = CGB_ST_INVALID;
      mu = __longlong_as_double(0x7ff8000000000000ll);
#pragma unroll
      for (int k = 0; k < DEG; ++k) z[k] = mk(mu, mu);
    }
    mag[i] = mu;
    if (status) status[i] = flags;
    if (mask_out) mask_out[i] = m;
  }
  if (images_out) {
    if (i < n) {
#pragma unroll
      for (int k = 0; k < DEG; ++k) stage[tid * DEG + k] = z[k];
    }
    __syncthreads();
    for (int j = tid; j < cnt * DEG; j += PS_THREADS) images_out[base * DEG + j] = stage[j];
  }
}

template <int PREC>
cudaError_t launch_mag_ps_p(const Lens &L, const double *w, double *mag, double *images_out, uint32_t *mask_out,
                            int64_t n, int itmax, uint32_t *status, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  dim3 grid((unsigned)((n + PS_THREADS - 1) / PS_THREADS));
  const cd *wc = reinterpret_cast<const cd *>(w);
  cd *im = reinterpret_cast<cd *>(images_out);
  if (L.n == 2)
    mag_ps_kernel<PREC, 2><<<grid, PS_THREADS, 0, stream>>>(L, wc, mag, im, mask_out, n, itmax, status);
  else if (L.n == 3)
    mag_ps_kernel<PREC, 3><<<grid, PS_THREADS, 0, stream>>>(L, wc, mag, im, mask_out, n, itmax, status);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

// Per-point pass of mag(): the hexadecapole magnification and the routing
// test for binary lenses; triple lenses route to the contour integral
// (lightcurve.py:226-227) unless triple_routing asks for the reference's
// triple hexadecapole with its triple proximity test (1: as written, 2: third
// lens at r3).  A non-finite source position gives NaN and CGB_ST_INVALID.
template <int PREC, int NL>
__global__ void __launch_bounds__(PS_THREADS) lc_points_kernel(Lens L, double q, const cd *__restrict__ w, double rho,
                                                               double *__restrict__ mag, uint8_t *__restrict__ route,
                                                               int64_t n, int itmax, uint32_t *__restrict__ status,
                                                               int triple_routing) {
  constexpr int DEG = NL * NL + 1;
  const int64_t i = (int64_t)blockIdx.x * PS_THREADS + threadIdx.x;
  if (i >= n) return;
  uint32_t flags = 0;
  cd wi = w[i];
  if (!isfinite(wi.x) || !isfinite(wi.y)) {
    mag[i] = __longlong_as_double(0x7ff8000000000000ll);
    route[i] = 0;
    if (status) status[i] = CGB_ST_INVALID;
    return;
  }
  wi.x += L.x_cm;
  // Triple lenses take the contour integral (lightcurve.py:226-227) unless
  // routed; for q < 0.01 the routing test is proximity & planetary
  // (lightcurve.py:216-224), so where the planetary test fails the point takes
  // the contour integral whatever its images give: neither the images nor the
  // hexadecapole are needed (the contour kernel writes mag).
  if ((NL == 3 && triple_routing == 0) || (NL == 2 && q < 0.01 && !planetary_test(L, wi, rho))) {
    mag[i] = 0.0;
    route[i] = 1;
    if (status) status[i] = 0;
    return;
  }
  cd z[DEG];
  uint32_t m = images<PREC, NL>(L, wi, z, itmax, flags);
  double mu_multi = 0.0, dmu = 0.0;
#pragma unroll 1
  for (int k = 0; k < DEG; ++k) {
    if (!((m >> k) & 1u)) continue;
    cd W[5];
    hexa::wk<NL>(L, z[k], W);
    double mu0, dq, dh;
    hexa::terms(W, rho, 0.0, mu0, dq, dh);  // mag() passes no u1 (lightcurve.py:215)
    mu_multi += fabs(mu0 + dq + dh);
    dmu += fabs(dq) + fabs(dh);
  }
  bool hex_ok;
  if constexpr (NL == 2) {
    hex_ok = proximity_test_binary(L, wi, z, m, rho, dmu);  // (q < 0.01: the planetary test passed above)
  } else {
    hex_ok = proximity_test_triple(L, wi, z, m, rho, dmu, triple_routing == 1);
  }
  mag[i] = mu_multi;
  route[i] = hex_ok ? 0 : 1;
  if (status) status[i] = flags;
}

template <int PREC>
cudaError_t launch_lc_points_p(const Lens &L, double q, const double *w, double rho, double *mag, uint8_t *route,
                               int64_t n, int itmax, uint32_t *status, int triple_routing, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  dim3 grid((unsigned)((n + PS_THREADS - 1) / PS_THREADS));
  const cd *wc = reinterpret_cast<const cd *>(w);
  if (L.n == 2)
    lc_points_kernel<PREC, 2><<<grid, PS_THREADS, 0, stream>>>(L, q, wc, rho, mag, route, n, itmax, status, 0);
  else if (L.n == 3)
    lc_points_kernel<PREC, 3><<<grid, PS_THREADS, 0, stream>>>(L, q, wc, rho, mag, route, n, itmax, status,
                                                               triple_routing);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

// ---- batched light curves ----
// Point i belongs to curve c with offsets[c] <= i < offsets[c+1]; its source is
// on the curve's rectilinear trajectory at times[i] (trajectory.py:152-155 with
// pi_E = 0): w = (u0 cos a + tau sin a) + i (-u0 sin a + tau cos a), tau = (t - t0)/tE.
__device__ __forceinline__ int64_t curve_of(const int64_t *offsets, int64_t ncurves, int64_t i) {
  int64_t lo = 0, hi = ncurves - 1;
  while (lo < hi) {
    int64_t mid = (lo + hi + 1) >> 1;
    if (offsets[mid] <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Per-point pass of batched mag(): images, hexadecapole, routing tests; points
// that need the contour integral are appended to the device work queue
// (qcount, qlist).  With GRAD, hexadecapole-routed points also write their
// cotangent-weighted gradient row grow[i][(s, q, rho, u1, u0, alpha, t0, tE)]
// (forward-mode tangents through the images and the multipole series); the
// contour kernel writes the rows of the queued points.  Curves with parameters
// out of the domain give NaN, CGB_ST_INVALID and a zero row.
// TPP: threads per polynomial (1, or a group of 8 lanes per point: forward
// only); with a group, every lane evaluates the point and lane 0 writes it.
template <int PREC, bool GRAD, int TPP>
__global__ void __launch_bounds__(PS_THREADS) lc_points_batched_kernel(
    const CurveDev *__restrict__ curves, const int64_t *__restrict__ offsets, const double *__restrict__ times,
    int64_t ncurves, int64_t n, double *__restrict__ mag, uint8_t *__restrict__ route, uint32_t *__restrict__ status,
    int itmax, unsigned long long *qcount, int64_t *qlist, const double *__restrict__ cot, double *grow) {
  static_assert(TPP == 1 || (TPP == 8 && !GRAD), "lane groups: forward only");
  const int64_t i = ((int64_t)blockIdx.x * PS_THREADS + threadIdx.x) / TPP;
  if (i >= n) return;  // whole groups: i is the same on every lane of a group
  const int gr = threadIdx.x & (TPP - 1);
  const bool writer = gr == 0;
  const int64_t c = curve_of(offsets, ncurves, i);
  const CurveDev cv = curves[c];
  if (!(cv.s > 0) || !(cv.q > 0) || !(cv.rho > 0) || !(cv.tE != 0) || !isfinite(cv.s) || !isfinite(cv.q) ||
      !isfinite(cv.rho) || !isfinite(cv.u1) || !isfinite(cv.u0) || !isfinite(cv.alpha) || !isfinite(cv.t0) ||
      !isfinite(cv.tE) || !isfinite(times[i])) {  // not evaluated: NaN, no gradient
    if (!writer) return;
    mag[i] = __longlong_as_double(0x7ff8000000000000ll);
    route[i] = 0;
    if (status) status[i] = CGB_ST_INVALID;
    if (GRAD) {
#pragma unroll
      for (int k = 0; k < 8; ++k) grow[i * 8 + k] = 0.0;
    }
    return;
  }
  const Lens L = make_lens(2, cv.s, cv.q, 0.0, 0.0, 0.0);
  const double tau = (times[i] - cv.t0) / cv.tE;
  double sa, ca;
  sincos(cv.alpha, &sa, &ca);
  const cd wi = mk(cv.u0 * ca + tau * sa + L.x_cm, -cv.u0 * sa + tau * ca);
  // for q < 0.01 the routing test is proximity & planetary (lightcurve.py:216-224):
  // where the planetary test fails the point takes the contour integral whatever
  // its images give, so it is queued without them (the contour kernel writes mag)
  if (cv.q < 0.01 && !planetary_test(L, wi, cv.rho)) {
    if (!writer) return;
    mag[i] = 0.0;
    route[i] = 1;
    if (status) status[i] = 0;
    qlist[atomicAdd(qcount, 1ull)] = i;
    return;
  }
  uint32_t flags = 0;
  cd z[5];
  uint32_t m;
  if constexpr (TPP == 1) {
    m = images<PREC, 2>(L, wi, z, itmax, flags);
  } else {
    const unsigned gmask = ((1u << TPP) - 1u) << ((threadIdx.x & 31) - gr);
    m = images_group<PREC, TPP>(L, wi, z, itmax, flags, gmask);
  }
  double mu_multi = 0.0, dmu = 0.0;
  cd W[5][5];
  double val[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    val[k] = 0.0;
    if (!((m >> k) & 1u)) continue;
    hexa::wk<2>(L, z[k], W[k]);
    double mu0, dq, dh;
    hexa::terms(W[k], cv.rho, 0.0, mu0, dq, dh);
    val[k] = mu0 + dq + dh;
    mu_multi += fabs(val[k]);
    dmu += fabs(dq) + fabs(dh);
  }
  bool hex_ok = proximity_test_binary(L, wi, z, m, cv.rho, dmu);
  // (q < 0.01: the planetary test passed above)
  if (!writer) return;
  mag[i] = mu_multi;
  route[i] = hex_ok ? 0 : 1;
  if (status) status[i] = flags;
  if (!hex_ok) {
    const unsigned long long slot = atomicAdd(qcount, 1ull);
    qlist[slot] = i;
    return;
  }
  if (!GRAD) return;
  // tangents along (a, e1, rho, Re w0, Im w0)
  const double a = L.r[0].x, e1 = L.eps[0], e2 = L.eps[1];
  double d[5];
  for (int dir = 0; dir < 5; ++dir) {
    const double da = dir == 0, de1 = dir == 1, drho = dir == 2;
    const cd dw0 = mk(dir == 3, dir == 4);
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      if (!((m >> k) & 1u)) continue;
      const cd zb = conj(z[k]);
      const cd u = crecip(zb - mk(a, 0)), v = crecip(zb + mk(a, 0));
      const cd lam = u * u * e1 + v * v * e2;
      const cd fa = u * u * e1 - v * v * e2, fe = u - v;
      const cd g = dw0 + fa * da + fe * de1;
      const cd dz = cdiv(g - lam * conj(g), mk(1.0 - norm2(lam), 0.0));
      cd dW[5];
      hexa::wk_tangent_binary(L, z[k], dz, da, de1, dW);
      double dmu0, ddq, ddh;
      hexa::terms_tangent(W[k], dW, cv.rho, drho, 0.0, dmu0, ddq, ddh);
      acc += (val[k] > 0 ? 1.0 : (val[k] < 0 ? -1.0 : 0.0)) * (dmu0 + ddq + ddh);
    }
    d[dir] = acc;
  }
  const double q = cv.q, opq = 1.0 + q, ah = 0.5 * cv.s;
  const double ds = 0.5 * d[0] + d[3] * (1.0 - q) / (2.0 * opq);
  const double dqq = -d[1] / (opq * opq) - d[3] * 2.0 * ah / (opq * opq);
  const double du0 = d[3] * ca - d[4] * sa;
  const double dal = d[3] * (-cv.u0 * sa + tau * ca) + d[4] * (-cv.u0 * ca - tau * sa);
  const double dt0 = -(d[3] * sa + d[4] * ca) / cv.tE;
  const double dtE = -tau * (d[3] * sa + d[4] * ca) / cv.tE;
  const double ct = cot ? cot[i] : 1.0;
  double *gp = grow + i * 8;
  gp[0] = ct * ds;
  gp[1] = ct * dqq;
  gp[2] = ct * d[2];
  gp[3] = 0.0;  // the hexadecapole of mag() takes no limb darkening (lightcurve.py:215)
  gp[4] = ct * du0;
  gp[5] = ct * dal;
  gp[6] = ct * dt0;
  gp[7] = ct * dtE;
}

template <int PREC>
cudaError_t launch_lc_points_batched_p(const EsParams &P, int64_t n, double *mag, uint8_t *route, uint32_t *status,
                                       unsigned long long *qcount, int64_t *qlist, bool grad, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  if (grad) {
    dim3 grid((unsigned)((n + PS_THREADS - 1) / PS_THREADS));
    lc_points_batched_kernel<PREC, true, 1><<<grid, PS_THREADS, 0, stream>>>(P.curves, P.offsets, P.times, P.ncurves, n,
                                                                             mag, route, status, P.itmax, qcount,
                                                                             qlist, P.cot, P.grow);
  } else if (P.point_lanes == 8) {
    dim3 grid((unsigned)((n * 8 + PS_THREADS - 1) / PS_THREADS));
    lc_points_batched_kernel<PREC, false, 8><<<grid, PS_THREADS, 0, stream>>>(P.curves, P.offsets, P.times, P.ncurves,
                                                                              n, mag, route, status, P.itmax, qcount,
                                                                              qlist, nullptr, nullptr);
  } else {
    dim3 grid((unsigned)((n + PS_THREADS - 1) / PS_THREADS));
    lc_points_batched_kernel<PREC, false, 1><<<grid, PS_THREADS, 0, stream>>>(P.curves, P.offsets, P.times, P.ncurves,
                                                                              n, mag, route, status, P.itmax, qcount,
                                                                              qlist, nullptr, nullptr);
  }
  return cudaGetLastError();
}

}  // namespace cgb
