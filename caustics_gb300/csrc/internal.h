// Host-side launchers shared between the translation units of the library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "lens.cuh"

namespace cgb {

enum Precision : int { FP64 = 0, MIXED = 1, FP64_COMP = 2 };

// lens-equation polynomial coefficients, low -> high (point_source.cu)
cudaError_t launch_lens_poly(const Lens &L, const double *w, double *coeffs, int64_t n, cudaStream_t stream);

cudaError_t launch_ea_solve(const double *coeffs, const double *roots_init, double *roots, int64_t n, int deg,
                            int itmax, int precision, uint32_t *status, cudaStream_t stream);

// implicit-function JVP / VJP of polynomial roots (roots_ad.cu)
cudaError_t launch_roots_jvp(const double *coeffs, const double *roots, const double *dcoeffs, double *droots,
                             int64_t n, int deg, cudaStream_t stream);
cudaError_t launch_roots_vjp(const double *coeffs, const double *roots, const double *ct_roots, double *ct_coeffs,
                             int64_t n, int deg, int conjugate, cudaStream_t stream);

// marginalised log-likelihood over (F_s, F_b), diagonal covariance (likelihood.cu)
cudaError_t launch_marg_ll(const int64_t *offsets, int64_t ncurves, const double *A, const double *fobs,
                           const double *C_inv, double *beta, double *ll, double *dll, const double *ll_cot,
                           cudaStream_t stream);

// annual-parallax trajectory (trajectory.cu)
cudaError_t launch_parallax(const double *t_jpl, const double *s_e, const double *s_n, const double *s_e_dot,
                            const double *s_n_dot, int64_t njpl, const double *t, int64_t n, double u0, double t0,
                            double tE, double piEE, double piEN, double *w, double *dw, cudaStream_t stream);

// critical curves and caustics (critical.cu)
size_t critical_workspace_bytes(int npts, int nlenses);
cudaError_t launch_critical(const Lens &L, int npts, int itmax, double *z_cr, double *z_ca, uint32_t *status,
                            void *ws, cudaStream_t stream);

cudaError_t launch_mag_ps(const Lens &L, const double *w, double *mag, double *images, uint32_t *image_mask,
                          int64_t n, int itmax, int precision, uint32_t *status, cudaStream_t stream);

// Light-curve point pass: images, hexadecapole, proximity (+ planetary when
// q < 0.01) tests.  Writes mu_multi (the hexadecapole magnification) into mag and
// route[i] = 1 where the full contour integration is needed.
cudaError_t launch_lc_points(const Lens &L, double q, const double *w, double rho, double *mag, uint8_t *route,
                             int64_t n, int itmax, int precision, uint32_t *status, int triple_routing,
                             cudaStream_t stream);

}  // namespace cgb
