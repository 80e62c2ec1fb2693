// Critical curves and caustics (the reference's critical_and_caustic_curves,
// src/caustics/point_source.py:1582-1649).
//
// On a critical curve det J = 0, i.e. sum_j eps_j / (z - r_j)^2 = e^{-i phi} for
// some phase phi (|lambda| = 1).  Clearing denominators gives the degree-2n
// polynomial
//   e^{-i phi} prod_j (z - r_j)^2 - sum_j eps_j prod_{k != j} (z - r_k)^2 = 0,
// solved for npts phases phi on linspace(-pi, pi, npts).  The roots of
// consecutive phases are chained into continuous curves by the reference's
// greedy nearest matching (utils.py:15-40 inside a lax.scan), the curves are
// mapped through the lens equation to the caustics, and both are shifted by
// the centre of mass.
//
// Kernels: one thread per phase solves its polynomial (FP64 Aberth; the first
// phase with the reference's iteration and real initial guesses, which fixes
// the curve labels); one thread per (phase, root) sorts the candidate roots of
// the next phase by distance (4 bits each in a 64-bit word); one CTA runs the
// integer chaining and writes the curves.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/caustics_gb300.h"
#include "aberth.cuh"
#include "aberth_ref.cuh"
#include "internal.h"
#include "lens.cuh"

namespace cgb {
namespace {

constexpr int CR_THREADS = 128;

template <int NL>
__device__ void critical_poly(const Lens &L, double phi, cd (&p)[2 * NL + 1]) {
  double sn, cs;
  sincos(phi, &sn, &cs);
  const cd x = mk(cs, -sn);  // e^{-i phi}
  // (z - r_j)^2 = r_j^2 - 2 r_j z + z^2, low -> high
  cd sq[NL][3];
#pragma unroll
  for (int j = 0; j < NL; ++j) {
    sq[j][0] = L.r[j] * L.r[j];
    sq[j][1] = L.r[j] * -2.0;
    sq[j][2] = mk(1.0, 0.0);
  }
  cd all[2 * NL + 1], rest[2 * NL - 1];
#pragma unroll
  for (int i = 0; i <= 2 * NL; ++i) all[i] = mk(i == 0 ? 1.0 : 0.0, 0.0);
#pragma unroll
  for (int i = 0; i < 2 * NL - 1; ++i) rest[i] = mk(0.0, 0.0);
#pragma unroll
  for (int j = 0; j < NL; ++j) {
    // all *= (z - r_j)^2
#pragma unroll
    for (int i = 2 * NL; i >= 0; --i) {
      cd acc = mk(0.0, 0.0);
#pragma unroll
      for (int m = 0; m < 3; ++m)
        if (i - m >= 0) acc = acc + all[i - m] * sq[j][m];
      all[i] = acc;
    }
    // rest += eps_j prod_{k != j} (z - r_k)^2
    cd t[2 * NL - 1];
#pragma unroll
    for (int i = 0; i < 2 * NL - 1; ++i) t[i] = mk(i == 0 ? L.eps[j] : 0.0, 0.0);
#pragma unroll
    for (int k = 0; k < NL; ++k) {
      if (k == j) continue;
#pragma unroll
      for (int i = 2 * NL - 2; i >= 0; --i) {
        cd acc = mk(0.0, 0.0);
#pragma unroll
        for (int m = 0; m < 3; ++m)
          if (i - m >= 0) acc = acc + t[i - m] * sq[k][m];
        t[i] = acc;
      }
    }
#pragma unroll
    for (int i = 0; i < 2 * NL - 1; ++i) rest[i] = rest[i] + t[i];
  }
#pragma unroll
  for (int i = 0; i <= 2 * NL; ++i) p[i] = x * all[i] - (i < 2 * NL - 1 ? rest[i] : mk(0.0, 0.0));
}

template <int NL>
__global__ void __launch_bounds__(CR_THREADS) critical_roots_kernel(Lens L, int npts, int itmax, cd *zraw,
                                                                    uint32_t *flags) {
  constexpr int DEG = 2 * NL;
  const int k = blockIdx.x * CR_THREADS + threadIdx.x;
  if (k >= npts) return;
  // numpy.linspace(-pi, pi, npts): start + k * step, the last point exactly pi
  const double pi = 3.141592653589793;
  const double step = (npts > 1) ? 2.0 * pi / (double)(npts - 1) : 0.0;
  const double phi = (k == npts - 1 && npts > 1) ? pi : __dadd_rn(__dmul_rn((double)k, step), -pi);
  cd p[DEG + 1], z[DEG];
  critical_poly<NL>(L, phi, p);
  int it;
  if (k == 0)
    it = refea::solve<DEG>(p, z, itmax, false);  // labels the curves as the reference's solver orders these roots
  else
    it = aberth64<DEG>(p, z, itmax, false);
  if (it < 0) atomicOr(flags, (uint32_t)CGB_ST_NOCONV);
#pragma unroll
  for (int i = 0; i < DEG; ++i) zraw[(size_t)k * DEG + i] = z[i];
}

// cand[k][r]: roots of phase k sorted by distance to root r of phase k-1
// (stable: ties keep the lower index, as the reference's argsort does).
template <int DEG>
__global__ void __launch_bounds__(CR_THREADS) critical_cand_kernel(const cd *zraw, int npts, uint64_t *cand) {
  const int64_t idx = (int64_t)blockIdx.x * CR_THREADS + threadIdx.x;
  if (idx >= (int64_t)(npts - 1) * DEG) return;
  const int k = 1 + (int)(idx / DEG), r = (int)(idx % DEG);
  const cd a = zraw[(size_t)(k - 1) * DEG + r];
  double d[DEG];
  int o[DEG];
#pragma unroll
  for (int j = 0; j < DEG; ++j) {
    d[j] = norm2(zraw[(size_t)k * DEG + j] - a);
    o[j] = j;
  }
  for (int i = 1; i < DEG; ++i) {  // insertion sort, stable
    const int oj = o[i];
    const double dj = d[oj];
    int m = i - 1;
    while (m >= 0 && d[o[m]] > dj) {
      o[m + 1] = o[m];
      --m;
    }
    o[m + 1] = oj;
  }
  uint64_t c = 0;
#pragma unroll
  for (int j = 0; j < DEG; ++j) c |= (uint64_t)o[j] << (4 * j);
  cand[(size_t)k * DEG + r] = c;
}

// One CTA: the chain of greedy matchings (integer work on one thread, the
// permutation of every phase kept in shared memory), then all threads write the
// curves z_cr[curve][phase] and z_ca = lens_eq(z_cr), both minus x_cm.
template <int NL>
__global__ void __launch_bounds__(256) critical_chain_kernel(Lens L, const cd *zraw, const uint64_t *cand, int npts,
                                                             cd *zcr, cd *zca) {
  constexpr int DEG = 2 * NL;
  extern __shared__ uint64_t perm[];  // [npts], 4 bits per curve: curve -> raw root
  if (threadIdx.x == 0) {
    uint64_t prev = 0;
    for (int i = 0; i < DEG; ++i) prev |= (uint64_t)i << (4 * i);
    perm[0] = prev;
    for (int k = 1; k < npts; ++k) {
      uint32_t taken = 0;
      uint64_t cur = 0;
      for (int i = 0; i < DEG; ++i) {
        const int r = (int)((prev >> (4 * i)) & 15u);
        const uint64_t c = cand[(size_t)k * DEG + r];
        int pick = 0;
        for (int t = 0; t < DEG; ++t) {
          const int j = (int)((c >> (4 * t)) & 15u);
          if (!((taken >> j) & 1u)) {
            pick = j;
            break;
          }
        }
        taken |= 1u << pick;
        cur |= (uint64_t)pick << (4 * i);
      }
      perm[k] = cur;
      prev = cur;
    }
  }
  __syncthreads();
  const cd shift = mk(L.x_cm, 0.0);
  for (int64_t idx = threadIdx.x; idx < (int64_t)npts * DEG; idx += blockDim.x) {
    const int i = (int)(idx / npts), k = (int)(idx % npts);
    const cd z = zraw[(size_t)k * DEG + (int)((perm[k] >> (4 * i)) & 15u)];
    zcr[idx] = z - shift;
    zca[idx] = lens_eq<NL>(L, z) - shift;
  }
}

}  // namespace

size_t critical_workspace_bytes(int npts, int nlenses) {
  const size_t deg = 2 * (size_t)nlenses;
  return (size_t)(npts > 0 ? npts : 0) * deg * (sizeof(cd) + sizeof(uint64_t)) + 16;
}

cudaError_t launch_critical(const Lens &L, int npts, int itmax, double *z_cr, double *z_ca, uint32_t *status,
                            void *ws, cudaStream_t stream) {
  const int deg = 2 * L.n;
  cd *zraw = reinterpret_cast<cd *>(ws);
  uint64_t *cand = reinterpret_cast<uint64_t *>(zraw + (size_t)npts * deg);
  uint32_t *flags = status ? status : reinterpret_cast<uint32_t *>(cand + (size_t)npts * deg);
  cudaError_t e = cudaMemsetAsync(flags, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  const unsigned g1 = (unsigned)((npts + CR_THREADS - 1) / CR_THREADS);
  const unsigned g2 = (unsigned)(((int64_t)(npts > 1 ? npts - 1 : 0) * deg + CR_THREADS - 1) / CR_THREADS);
  const size_t smem = sizeof(uint64_t) * (size_t)npts;
  if (L.n == 2) {
    critical_roots_kernel<2><<<g1, CR_THREADS, 0, stream>>>(L, npts, itmax, zraw, flags);
    if (g2) critical_cand_kernel<4><<<g2, CR_THREADS, 0, stream>>>(zraw, npts, cand);
    e = cudaFuncSetAttribute(critical_chain_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    critical_chain_kernel<2><<<1, 256, smem, stream>>>(L, zraw, cand, npts, (cd *)z_cr, (cd *)z_ca);
  } else {
    critical_roots_kernel<3><<<g1, CR_THREADS, 0, stream>>>(L, npts, itmax, zraw, flags);
    if (g2) critical_cand_kernel<6><<<g2, CR_THREADS, 0, stream>>>(zraw, npts, cand);
    e = cudaFuncSetAttribute(critical_chain_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    critical_chain_kernel<3><<<1, 256, smem, stream>>>(L, zraw, cand, npts, (cd *)z_cr, (cd *)z_ca);
  }
  return cudaGetLastError();
}

}  // namespace cgb
