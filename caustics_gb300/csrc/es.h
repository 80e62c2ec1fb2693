// Extended-source kernel parameters (shared by the launchers and the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "lens.cuh"

namespace cgb {

constexpr int GL_MAX = 64;  // Gauss-Legendre nodes per half interval

struct EsParams {
  Lens L;
  double rho, u1;
  int n0;      // initial limb points, int(npts/2)
  int n_add;   // points added per refinement round, int(int(npts/2)/niter)
  int niter;   // refinement rounds (10 in the reference)
  int Lcap;    // n0 + niter * n_add
  int CPcap;   // contour point capacity
  int ld;      // limb darkening on
  int n1, n2;  // Gauss-Legendre nodes on [a, split] and [split, b] (npts_ld/2 and the rest)
  int itmax;
  double *dbg;  // optional per-point diagnostics (cgb_debug_extended_source), stride ES_DBG_STRIDE(Lcap)
  double gl_x[2][GL_MAX], gl_w[2][GL_MAX];
};

// diagnostics record: [L, ncont, flags, (start, count, parity, integral) x 13, theta[0..L)]
#define ES_DBG_HEAD (3 + 4 * 13)
#define ES_DBG_STRIDE(lcap) (ES_DBG_HEAD + (lcap))

size_t es_smem_bytes(const EsParams &P, int nl);

cudaError_t launch_es(const EsParams &P, const double *w0, const int64_t *index, int64_t n, double *mag,
                      uint32_t *status, int precision, int grid, cudaStream_t stream);

// Only the points with route[i] != 0 are integrated; status is OR-ed in.
cudaError_t launch_es_routed(const EsParams &P, const double *w0, const uint8_t *route, int64_t n, double *mag,
                             uint32_t *status, int precision, int grid, cudaStream_t stream);

// Gauss-Legendre nodes/weights on [-1, 1], ascending (host)
void gauss_legendre(int n, double *x, double *w);

}  // namespace cgb
