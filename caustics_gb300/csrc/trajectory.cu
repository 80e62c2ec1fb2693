// Source trajectory with annual parallax (the reference's
// AnnualParallaxTrajectory.compute, src/caustics/trajectory.py:106-157):
//   ds = s(t) - s(t0) - (t - t0) sdot(t0)   (projected Sun position, east and
//        north, linearly interpolated in the ephemeris table as jnp.interp,
//        clamped outside it),
//   psi = atan2(piEE, piEN), piE = |(piEE, piEN)|,
//   w = [u0 cos psi + tau sin psi + piE ds_e] + i [-u0 sin psi + tau cos psi + piE ds_n],
//   tau = (t - t0) / tE.
// One thread per time; optional Jacobian dw / d(u0, t0, tE, piEE, piEN), the
// piecewise-linear interpolation differentiated segment by segment.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "cplx.cuh"
#include "internal.h"

namespace cgb {
namespace {

constexpr int TR_THREADS = 256;

// value and slope of the piecewise-linear interpolant (jnp.interp: clamped)
__device__ __forceinline__ void interp(const double *xp, const double *fp, int64_t n, double x, double &f,
                                       double &slope) {
  if (x <= xp[0]) {
    f = fp[0];
    slope = 0.0;
    return;
  }
  if (x >= xp[n - 1]) {
    f = fp[n - 1];
    slope = 0.0;
    return;
  }
  int64_t lo = 0, hi = n - 1;  // xp[lo] < x < xp[hi]
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (xp[mid] <= x) lo = mid; else hi = mid;
  }
  slope = (fp[hi] - fp[lo]) / (xp[hi] - xp[lo]);
  f = fp[lo] + (x - xp[lo]) * slope;
}

__global__ void __launch_bounds__(TR_THREADS) parallax_kernel(const double *__restrict__ tj,
                                                              const double *__restrict__ se,
                                                              const double *__restrict__ sn,
                                                              const double *__restrict__ sed,
                                                              const double *__restrict__ snd, int64_t nj,
                                                              const double *__restrict__ t, int64_t n, double u0,
                                                              double t0, double tE, double piEE, double piEN, cd *w,
                                                              cd *dw) {
  const int64_t i = (int64_t)blockIdx.x * TR_THREADS + threadIdx.x;
  if (i >= n) return;
  const double ti = t[i];
  double fe, ge, fn, gn, fe0, ge0, fn0, gn0, de0, hde, dn0, hdn;
  interp(tj, se, nj, ti, fe, ge);
  interp(tj, sn, nj, ti, fn, gn);
  interp(tj, se, nj, t0, fe0, ge0);
  interp(tj, sn, nj, t0, fn0, gn0);
  interp(tj, sed, nj, t0, de0, hde);
  interp(tj, snd, nj, t0, dn0, hdn);
  const double dt = ti - t0;
  const double dse = fe - fe0 - dt * de0, dsn = fn - fn0 - dt * dn0;
  const double psi = atan2(piEE, piEN), piE = sqrt(piEN * piEN + piEE * piEE);
  double sp, cp;
  sincos(psi, &sp, &cp);
  const double tau = dt / tE;
  w[i] = mk(u0 * cp + tau * sp + piE * dse, -u0 * sp + tau * cp + piE * dsn);
  if (dw) {
    cd *J = dw + 5 * i;
    J[0] = mk(cp, -sp);  // d/du0
    // d/dt0: tau' = -1/tE, ds' = -s'(t0) + sdot(t0) - (t - t0) sdot'(t0)
    const double dse_t0 = -ge0 + de0 - dt * hde, dsn_t0 = -gn0 + dn0 - dt * hdn;
    J[1] = mk(-sp / tE + piE * dse_t0, -cp / tE + piE * dsn_t0);
    J[2] = mk(-tau / tE * sp, -tau / tE * cp);  // d/dtE
    // psi and piE in terms of (piEE, piEN): dpsi/dpiEE = piEN/piE^2, dpsi/dpiEN = -piEE/piE^2
    const double ip2 = 1.0 / (piE * piE);
    const double dw_dpsi_x = -u0 * sp + tau * cp, dw_dpsi_y = -u0 * cp - tau * sp;
    J[3] = mk(dw_dpsi_x * piEN * ip2 + piEE / piE * dse, dw_dpsi_y * piEN * ip2 + piEE / piE * dsn);
    J[4] = mk(-dw_dpsi_x * piEE * ip2 + piEN / piE * dse, -dw_dpsi_y * piEE * ip2 + piEN / piE * dsn);
  }
}

}  // namespace

cudaError_t launch_parallax(const double *t_jpl, const double *s_e, const double *s_n, const double *s_e_dot,
                            const double *s_n_dot, int64_t njpl, const double *t, int64_t n, double u0, double t0,
                            double tE, double piEE, double piEN, double *w, double *dw, cudaStream_t stream) {
  parallax_kernel<<<(unsigned)((n + TR_THREADS - 1) / TR_THREADS), TR_THREADS, 0, stream>>>(
      t_jpl, s_e, s_n, s_e_dot, s_n_dot, njpl, t, n, u0, t0, tE, piEE, piEN, (cd *)w, (cd *)dw);
  return cudaGetLastError();
}

}  // namespace cgb
