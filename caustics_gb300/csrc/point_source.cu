// Host launchers of the point-source kernels (point_source.cuh): select the
// per-precision instantiation (ps_fp64.cu, ps_mixed.cu, ps_comp.cu) from the
// runtime precision.  The light-curve point passes only take FP64 or MIXED.
// Also two precision-free kernels: the lens-equation polynomial of source
// positions, and the per-curve sums of the batched adjoint's point rows.
#include "aberth.cuh"
#include "es.h"
#include "internal.h"

namespace cgb {

template <int PREC>
cudaError_t launch_ea_solve_p(const double *coeffs, const double *roots_init, double *roots, int64_t n, int deg,
                              int itmax, uint32_t *status, cudaStream_t stream);
template <int PREC>
cudaError_t launch_mag_ps_p(const Lens &L, const double *w, double *mag, double *images_out, uint32_t *mask_out,
                            int64_t n, int itmax, uint32_t *status, cudaStream_t stream);
template <int PREC>
cudaError_t launch_lc_points_p(const Lens &L, double q, const double *w, double rho, double *mag, uint8_t *route,
                               int64_t n, int itmax, uint32_t *status, int triple_routing, cudaStream_t stream);
template <int PREC>
cudaError_t launch_lc_points_batched_p(const EsParams &P, int64_t n, double *mag, uint8_t *route, uint32_t *status,
                                       unsigned long long *qcount, int64_t *qlist, bool grad, cudaStream_t stream);

constexpr int AUX_THREADS = 128;

// The per-point pass of triple-lens light curves: the reference's mag() sends
// every triple-lens point to the contour integral (src/caustics/lightcurve.py:
// 226-227), so a point is checked and queued; the contour kernel writes mag.
__global__ void __launch_bounds__(AUX_THREADS)
    lc_points_batched_triple_kernel(const CurveDev3 *__restrict__ curves, const int64_t *__restrict__ offsets,
                                    const double *__restrict__ times, int64_t ncurves, int64_t n,
                                    double *__restrict__ mag, uint8_t *__restrict__ route,
                                    uint32_t *__restrict__ status, unsigned long long *qcount, int64_t *qlist,
                                    double *__restrict__ grow) {
  const int64_t i = (int64_t)blockIdx.x * AUX_THREADS + threadIdx.x;
  if (i >= n) return;
  int64_t lo = 0, hi = ncurves - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (offsets[mid] <= i) lo = mid; else hi = mid - 1;
  }
  const CurveDev3 cv = curves[lo];
  const bool ok = cv.s > 0 && cv.q > 0 && cv.q3 >= 0 && cv.rho > 0 && cv.tE != 0 && isfinite(cv.s) &&
                  isfinite(cv.q) && isfinite(cv.q3) && isfinite(cv.r3) && isfinite(cv.psi) && isfinite(cv.rho) &&
                  isfinite(cv.u1) && isfinite(cv.u0) && isfinite(cv.alpha) && isfinite(cv.t0) && isfinite(cv.tE) &&
                  isfinite(times[i]);
  if (!ok) {  // not evaluated: NaN, no gradient
    mag[i] = __longlong_as_double(0x7ff8000000000000ll);
    route[i] = 0;
    if (status) status[i] = CGB_ST_INVALID;
    if (grow) {
#pragma unroll
      for (int k = 0; k < 11; ++k) grow[i * 11 + k] = 0.0;
    }
    return;
  }
  mag[i] = 0.0;
  route[i] = 1;
  if (status) status[i] = 0;
  qlist[atomicAdd(qcount, 1ull)] = i;
}

cudaError_t launch_lc_points_batched_triple(const EsParams &P, int64_t n, double *mag, uint8_t *route,
                                            uint32_t *status, unsigned long long *qcount, int64_t *qlist,
                                            cudaStream_t stream, double *grow) {
  if (n == 0) return cudaSuccess;
  lc_points_batched_triple_kernel<<<(unsigned)((n + AUX_THREADS - 1) / AUX_THREADS), AUX_THREADS, 0, stream>>>(
      P.curves3, P.offsets, P.times, P.ncurves, n, mag, route, status, qcount, qlist, grow);
  return cudaGetLastError();
}

// cgrad[c][k] = sum of the rows grow[i][k] of curve c's points: one warp per
// curve, each lane summing a fixed stride of points, then a fixed shuffle tree,
// so repeated calls give identical bits.  NC: the columns of a row (8
// binary-lens curve parameters, 11 triple-lens).
template <int NC>
__global__ void __launch_bounds__(AUX_THREADS)
    curve_grad_reduce_kernel(const int64_t *__restrict__ offsets, int64_t ncurves, const double *__restrict__ grow,
                             double *__restrict__ cgrad) {
  const int64_t c = (int64_t)blockIdx.x * (AUX_THREADS / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= ncurves) return;
  const int64_t b = offsets[c], e = offsets[c + 1];
  double acc[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) acc[k] = 0.0;
  for (int64_t i = b + lane; i < e; i += 32) {
#pragma unroll
    for (int k = 0; k < NC; ++k) acc[k] += grow[i * NC + k];
  }
#pragma unroll
  for (int k = 0; k < NC; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
  }
  if (lane < NC) {
    double v = acc[0];
#pragma unroll
    for (int k = 1; k < NC; ++k) v = lane == k ? acc[k] : v;
    cgrad[c * NC + lane] = v;
  }
}

cudaError_t launch_curve_grad_reduce(const int64_t *offsets, int64_t ncurves, const double *grow, double *cgrad,
                                     cudaStream_t stream, int ncols) {
  if (ncurves == 0) return cudaSuccess;
  constexpr int per_block = AUX_THREADS / 32;
  const unsigned grid = (unsigned)((ncurves + per_block - 1) / per_block);
  if (ncols == 11)
    curve_grad_reduce_kernel<11><<<grid, AUX_THREADS, 0, stream>>>(offsets, ncurves, grow, cgrad);
  else
    curve_grad_reduce_kernel<8><<<grid, AUX_THREADS, 0, stream>>>(offsets, ncurves, grow, cgrad);
  return cudaGetLastError();
}

// Lens-equation polynomial of each source position (user frame; shifted by
// x_cm as mag_point_source does), low -> high: one thread per position.
template <int NL>
__global__ void __launch_bounds__(AUX_THREADS) lens_poly_kernel(Lens L, const cd *__restrict__ w,
                                                                cd *__restrict__ coeffs, int64_t n) {
  constexpr int DEG = NL * NL + 1;
  const int64_t i = (int64_t)blockIdx.x * AUX_THREADS + threadIdx.x;
  if (i >= n) return;
  const cd wi = mk(w[i].x + L.x_cm, w[i].y);
  cd p[DEG + 1];
  lens_poly<NL>(L, wi, p);
#pragma unroll
  for (int k = 0; k <= DEG; ++k) coeffs[i * (DEG + 1) + k] = p[k];
}

cudaError_t launch_lens_poly(const Lens &L, const double *w, double *coeffs, int64_t n, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  const unsigned grid = (unsigned)((n + AUX_THREADS - 1) / AUX_THREADS);
  const cd *wc = reinterpret_cast<const cd *>(w);
  cd *c = reinterpret_cast<cd *>(coeffs);
  if (L.n == 2)
    lens_poly_kernel<2><<<grid, AUX_THREADS, 0, stream>>>(L, wc, c, n);
  else if (L.n == 3)
    lens_poly_kernel<3><<<grid, AUX_THREADS, 0, stream>>>(L, wc, c, n);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_ea_solve(const double *coeffs, const double *roots_init, double *roots, int64_t n, int deg,
                            int itmax, int precision, uint32_t *status, cudaStream_t stream) {
  switch (precision) {
    case FP64: return launch_ea_solve_p<FP64>(coeffs, roots_init, roots, n, deg, itmax, status, stream);
    case MIXED: return launch_ea_solve_p<MIXED>(coeffs, roots_init, roots, n, deg, itmax, status, stream);
    case FP64_COMP: return launch_ea_solve_p<FP64_COMP>(coeffs, roots_init, roots, n, deg, itmax, status, stream);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_mag_ps(const Lens &L, const double *w, double *mag, double *images_out, uint32_t *mask_out,
                          int64_t n, int itmax, int precision, uint32_t *status, cudaStream_t stream) {
  switch (precision) {
    case FP64: return launch_mag_ps_p<FP64>(L, w, mag, images_out, mask_out, n, itmax, status, stream);
    case MIXED: return launch_mag_ps_p<MIXED>(L, w, mag, images_out, mask_out, n, itmax, status, stream);
    case FP64_COMP: return launch_mag_ps_p<FP64_COMP>(L, w, mag, images_out, mask_out, n, itmax, status, stream);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_lc_points(const Lens &L, double q, const double *w, double rho, double *mag, uint8_t *route,
                             int64_t n, int itmax, int precision, uint32_t *status, int triple_routing,
                             cudaStream_t stream) {
  switch (precision) {
    case FP64: return launch_lc_points_p<FP64>(L, q, w, rho, mag, route, n, itmax, status, triple_routing, stream);
    case MIXED: return launch_lc_points_p<MIXED>(L, q, w, rho, mag, route, n, itmax, status, triple_routing, stream);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_lc_points_batched(const EsParams &P, int64_t n, double *mag, uint8_t *route, uint32_t *status,
                                     int precision, unsigned long long *qcount, int64_t *qlist, bool grad,
                                     cudaStream_t stream) {
  switch (precision) {
    case FP64: return launch_lc_points_batched_p<FP64>(P, n, mag, route, status, qcount, qlist, grad, stream);
    case MIXED: return launch_lc_points_batched_p<MIXED>(P, n, mag, route, status, qcount, qlist, grad, stream);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace cgb
