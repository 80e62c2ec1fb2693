// Implicit-function derivatives of polynomial roots, the reference's JVP rule
// for its root-solver primitive (src/caustics/ehrlich_aberth_primitive.py:252-312):
// for p(z_r) = 0 with coefficients p_k (low -> high),
//   dz_r = -sum_k z_r^k dp_k / p'(z_r).
// The VJP is the transpose of that linear map (JAX's convention for a
// holomorphic map) or its conjugate transpose (torch's convention for complex
// tensors).  FP64 throughout; one thread per root (JVP) or per coefficient (VJP),
// so any degree works without templates.
#include <cuda_runtime.h>
#include <stdint.h>

#include "cplx.cuh"
#include "internal.h"

namespace cgb {
namespace {

constexpr int AD_THREADS = 256;

// p'(z) by Horner on the derivative's coefficients k p_k.
__device__ __forceinline__ cd dpoly(const cd *p, int deg, cd z) {
  cd acc = p[deg] * (double)deg;
  for (int k = deg - 1; k >= 1; --k) acc = acc * z + p[k] * (double)k;
  return acc;
}

__global__ void __launch_bounds__(AD_THREADS) roots_jvp_kernel(const cd *__restrict__ p, const cd *__restrict__ z,
                                                               const cd *__restrict__ dp, cd *__restrict__ dz,
                                                               int64_t n, int deg) {
  const int64_t i = (int64_t)blockIdx.x * AD_THREADS + threadIdx.x;  // root index
  if (i >= n * deg) return;
  const int64_t m = i / deg;
  const cd *pm = p + m * (deg + 1), *dpm = dp + m * (deg + 1);
  const cd zr = z[i];
  cd num = dpm[deg];  // sum_k dp_k z^k by Horner
  for (int k = deg - 1; k >= 0; --k) num = num * zr + dpm[k];
  dz[i] = -cdiv(num, dpoly(pm, deg, zr));
}

__global__ void __launch_bounds__(AD_THREADS) roots_vjp_kernel(const cd *__restrict__ p, const cd *__restrict__ z,
                                                               const cd *__restrict__ ct, cd *__restrict__ cp,
                                                               int64_t n, int deg, int conjugate) {
  const int64_t i = (int64_t)blockIdx.x * AD_THREADS + threadIdx.x;  // coefficient index
  if (i >= n * (deg + 1)) return;
  const int64_t m = i / (deg + 1);
  const int k = (int)(i - m * (deg + 1));
  const cd *pm = p + m * (deg + 1);
  cd acc = mk(0.0, 0.0);
  for (int r = 0; r < deg; ++r) {
    const cd zr = z[m * deg + r];
    cd zk = mk(1.0, 0.0);
    for (int j = 0; j < k; ++j) zk = zk * zr;
    cd d = -cdiv(zk, dpoly(pm, deg, zr));  // d z_r / d p_k
    if (conjugate) d = conj(d);
    acc = acc + d * ct[m * deg + r];
  }
  cp[i] = acc;
}

}  // namespace

cudaError_t launch_roots_jvp(const double *coeffs, const double *roots, const double *dcoeffs, double *droots,
                             int64_t n, int deg, cudaStream_t stream) {
  const int64_t work = n * deg;
  roots_jvp_kernel<<<(unsigned)((work + AD_THREADS - 1) / AD_THREADS), AD_THREADS, 0, stream>>>(
      (const cd *)coeffs, (const cd *)roots, (const cd *)dcoeffs, (cd *)droots, n, deg);
  return cudaGetLastError();
}

cudaError_t launch_roots_vjp(const double *coeffs, const double *roots, const double *ct_roots, double *ct_coeffs,
                             int64_t n, int deg, int conjugate, cudaStream_t stream) {
  const int64_t work = n * (deg + 1);
  roots_vjp_kernel<<<(unsigned)((work + AD_THREADS - 1) / AD_THREADS), AD_THREADS, 0, stream>>>(
      (const cd *)coeffs, (const cd *)roots, (const cd *)ct_roots, (cd *)ct_coeffs, n, deg, conjugate);
  return cudaGetLastError();
}

}  // namespace cgb
