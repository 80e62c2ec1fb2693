// Extended-source dispatch (src/caustics/extended_source.py:741-904): picks the
// kernel variant for the lens multiplicity and the precision.  The kernel
// itself is in es_kernel.cuh; each variant is compiled in its own translation
// unit (es_b64.cu, es_b32.cu, es_t64.cu, es_t32.cu; the adjoints es_b64g.cu,
// es_b32g.cu, es_t64g.cu, es_t32g.cu).
#include "es.h"
#include "internal.h"
#include "es_kernel.cuh"

namespace cgb {

template <int NL, int PREC, bool GRAD>
cudaError_t launch_es_variant(const EsParams &P, const cd *w0, const int64_t *index, const uint8_t *route, int64_t n,
                              double *mag, uint32_t *status, int grid, cudaStream_t stream);
extern template cudaError_t launch_es_variant<2, FP64, false>(const EsParams &, const cd *, const int64_t *, const uint8_t *,
                                                       int64_t, double *, uint32_t *, int, cudaStream_t);
extern template cudaError_t launch_es_variant<2, MIXED, false>(const EsParams &, const cd *, const int64_t *, const uint8_t *,
                                                        int64_t, double *, uint32_t *, int, cudaStream_t);
extern template cudaError_t launch_es_variant<3, FP64, false>(const EsParams &, const cd *, const int64_t *, const uint8_t *,
                                                       int64_t, double *, uint32_t *, int, cudaStream_t);
extern template cudaError_t launch_es_variant<3, MIXED, false>(const EsParams &, const cd *, const int64_t *, const uint8_t *,
                                                        int64_t, double *, uint32_t *, int, cudaStream_t);

extern template cudaError_t launch_es_variant<2, FP64, true>(const EsParams &, const cd *, const int64_t *,
                                                             const uint8_t *, int64_t, double *, uint32_t *, int,
                                                             cudaStream_t);
extern template cudaError_t launch_es_variant<2, MIXED, true>(const EsParams &, const cd *, const int64_t *,
                                                              const uint8_t *, int64_t, double *, uint32_t *, int,
                                                              cudaStream_t);
extern template cudaError_t launch_es_variant<3, FP64, true>(const EsParams &, const cd *, const int64_t *,
                                                             const uint8_t *, int64_t, double *, uint32_t *, int,
                                                             cudaStream_t);
extern template cudaError_t launch_es_variant<3, MIXED, true>(const EsParams &, const cd *, const int64_t *,
                                                              const uint8_t *, int64_t, double *, uint32_t *, int,
                                                              cudaStream_t);

static cudaError_t dispatch_es(const EsParams &P, const double *w0, const int64_t *index, const uint8_t *route,
                               int64_t n, double *mag, uint32_t *status, int precision, int grid,
                               cudaStream_t stream) {
  if (n == 0 && !P.qhead) return cudaSuccess;
  const cd *w = reinterpret_cast<const cd *>(w0);
  const int nl = P.curves3 ? 3 : (P.curves ? 2 : P.L.n);
  if (nl == 2)
    return precision == MIXED ? launch_es_variant<2, MIXED, false>(P, w, index, route, n, mag, status, grid, stream)
                              : launch_es_variant<2, FP64, false>(P, w, index, route, n, mag, status, grid, stream);
  if (nl == 3)
    return precision == MIXED ? launch_es_variant<3, MIXED, false>(P, w, index, route, n, mag, status, grid, stream)
                              : launch_es_variant<3, FP64, false>(P, w, index, route, n, mag, status, grid, stream);
  return cudaErrorInvalidValue;
}

cudaError_t launch_es(const EsParams &P, const double *w0, const int64_t *index, int64_t n, double *mag,
                      uint32_t *status, int precision, int grid, cudaStream_t stream) {
  return dispatch_es(P, w0, index, nullptr, n, mag, status, precision, grid, stream);
}

cudaError_t launch_es_routed(const EsParams &P, const double *w0, const uint8_t *route, int64_t n, double *mag,
                             uint32_t *status, int precision, int grid, cudaStream_t stream) {
  return dispatch_es(P, w0, nullptr, route, n, mag, status, precision, grid, stream);
}

cudaError_t launch_es_grad(const EsParams &P, const double *w0, const uint8_t *route, int64_t n, double *mag,
                           uint32_t *status, int precision, int grid, cudaStream_t stream) {
  if (n == 0 && !P.qhead) return cudaSuccess;
  const cd *w = reinterpret_cast<const cd *>(w0);
  const int nl = P.curves3 ? 3 : (P.curves ? 2 : P.L.n);
  if (nl == 3)
    return precision == MIXED ? launch_es_variant<3, MIXED, true>(P, w, nullptr, route, n, mag, status, grid, stream)
                              : launch_es_variant<3, FP64, true>(P, w, nullptr, route, n, mag, status, grid, stream);
  if (nl != 2) return cudaErrorInvalidValue;
  return precision == MIXED ? launch_es_variant<2, MIXED, true>(P, w, nullptr, route, n, mag, status, grid, stream)
                            : launch_es_variant<2, FP64, true>(P, w, nullptr, route, n, mag, status, grid, stream);
}

size_t es_smem_bytes(const EsParams &P, int nl, bool grad) {
  // must follow the layout in es_kernel (es_kernel.cuh)
  const int deg = nl * nl + 1;
  auto up16 = [](size_t v) { return (v + 15) / 16 * 16; };
  size_t live = 0;
  live += sizeof(cd) * (size_t)P.Lcap * deg;
  live += sizeof(double) * P.Lcap;
  live += sizeof(uint32_t) * (size_t)P.CPcap;
  live = up16(live);
  size_t dead = 0;
  dead += sizeof(double) * P.Lcap;
  dead += sizeof(uint64_t) * P.Lcap * (3 + deg);
  dead += (sizeof(MergeState) + 15) / 16 * 16;
  dead += sizeof(int) * (P.Lcap + 1);
  dead += sizeof(uint16_t) * P.Lcap * 5;
  dead = up16(live + dead) - live;
  const size_t gg = sizeof(cd) * (size_t)P.CPcap;
  size_t b = live + dead;
  if (grad && dead < gg) b += gg;  // the adjoint's accumulators reuse the dead region when it is large enough
  return up16(b);
}

}  // namespace cgb
