// Log-likelihood of light curves marginalised over the linear flux
// parameters beta = (F_s, F_b), diagonal data covariance (the reference's
// marginalized_log_likelihood, src/caustics/linalg.py:10-94, first branch).
//
// Per curve with magnifications A_i, fluxes f_i and inverse variances c_i:
//   F = M^T C M = [[sum c A^2, sum c A], [sum c A, sum c]],  Sigma = F^-1,
//   beta = Sigma [sum c A f, sum c f],  r_i = f_i - beta_0 A_i - beta_1,
//   ll = -1/2 sum c r^2 + 1/2 log det(2 pi Sigma).
// Because beta minimises chi^2, the gradient with respect to the
// magnifications only sees beta's explicit appearance and Sigma:
//   d ll / d A_i = c_i (r_i beta_0 - A_i Sigma_00 - Sigma_01).
// One CTA per curve (grid-stride over curves): pass 1 reduces the five moments
// in FP64, one thread solves the 2x2 system, pass 2 forms chi^2 and the
// gradient.  The curve's 24 B per point are read twice; the second read is
// served by L2 for any curve shorter than a few million points.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "internal.h"

namespace cgb {
namespace {

constexpr int LL_THREADS = 256;
constexpr int LL_WARPS = LL_THREADS / 32;

template <int N>
__device__ void block_sum(double (&v)[N], double (*red)[N]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; ++k) red[warp][k] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; ++k) {
    double s = 0.0;
    for (int w = 0; w < LL_WARPS; ++w) s += red[w][k];
    v[k] = s;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(LL_THREADS) marg_ll_kernel(const int64_t *__restrict__ offsets, int64_t ncurves,
                                                             const double *__restrict__ A,
                                                             const double *__restrict__ f,
                                                             const double *__restrict__ c, double *beta, double *ll,
                                                             double *dll, const double *__restrict__ ll_cot) {
  __shared__ double red5[LL_WARPS][5];
  __shared__ double red1[LL_WARPS][1];
  for (int64_t cu = blockIdx.x; cu < ncurves; cu += gridDim.x) {
    const int64_t lo = offsets[cu], hi = offsets[cu + 1];
    double m[5] = {0.0, 0.0, 0.0, 0.0, 0.0};  // c A^2, c A, c, c A f, c f
    for (int64_t i = lo + threadIdx.x; i < hi; i += LL_THREADS) {
      const double a = A[i], ci = c[i], fi = f[i];
      const double ca = ci * a;
      m[0] = fma(ca, a, m[0]);
      m[1] += ca;
      m[2] += ci;
      m[3] = fma(ca, fi, m[3]);
      m[4] = fma(ci, fi, m[4]);
    }
    block_sum<5>(m, red5);
    const double det = m[0] * m[2] - m[1] * m[1];
    const double s00 = m[2] / det, s01 = -m[1] / det, s11 = m[0] / det;  // Sigma = F^-1
    const double b0 = s00 * m[3] + s01 * m[4], b1 = s01 * m[3] + s11 * m[4];
    const bool ok = det > 0.0 && isfinite(det);
    const double w = ll_cot ? ll_cot[cu] : 1.0;
    double chi[1] = {0.0};
    for (int64_t i = lo + threadIdx.x; i < hi; i += LL_THREADS) {
      const double a = A[i], ci = c[i];
      const double r = f[i] - fma(b0, a, b1);
      chi[0] = fma(ci * r, r, chi[0]);
      if (dll) dll[i] = ok ? w * ci * (r * b0 - a * s00 - s01) : NAN;
    }
    block_sum<1>(chi, red1);
    if (threadIdx.x == 0) {
      const double two_pi = 6.283185307179586;
      // log det(2 pi Sigma) = 2 log(2 pi) - log det F
      const double val = -0.5 * chi[0] + 0.5 * (2.0 * log(two_pi) - log(det));
      ll[cu] = ok ? val : NAN;
      if (beta) {
        beta[2 * cu] = ok ? b0 : NAN;
        beta[2 * cu + 1] = ok ? b1 : NAN;
      }
    }
  }
}

}  // namespace

cudaError_t launch_marg_ll(const int64_t *offsets, int64_t ncurves, const double *A, const double *fobs,
                           const double *C_inv, double *beta, double *ll, double *dll, const double *ll_cot,
                           cudaStream_t stream) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t cap = (int64_t)(sms > 0 ? sms : 1) * 8;
  const unsigned grid = (unsigned)(ncurves < cap ? ncurves : cap);
  marg_ll_kernel<<<grid, LL_THREADS, 0, stream>>>(offsets, ncurves, A, fobs, C_inv, beta, ll, dll, ll_cot);
  return cudaGetLastError();
}

}  // namespace cgb
