// Host launchers of the point-source kernels (point_source.cuh): select the
// per-precision instantiation (ps_fp64.cu, ps_mixed.cu, ps_comp.cu) from the
// runtime precision.  The light-curve point passes only take FP64 or MIXED.
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
                               int64_t n, int itmax, uint32_t *status, cudaStream_t stream);
template <int PREC>
cudaError_t launch_lc_points_batched_p(const EsParams &P, int64_t n, double *mag, uint8_t *route, uint32_t *status,
                                       unsigned long long *qcount, int64_t *qlist, bool grad, cudaStream_t stream);

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
                             int64_t n, int itmax, int precision, uint32_t *status, cudaStream_t stream) {
  switch (precision) {
    case FP64: return launch_lc_points_p<FP64>(L, q, w, rho, mag, route, n, itmax, status, stream);
    case MIXED: return launch_lc_points_p<MIXED>(L, q, w, rho, mag, route, n, itmax, status, stream);
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
