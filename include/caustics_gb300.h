/*
 * caustics_gb300 — C ABI of the GB300 (sm_103a) magnification library.
 *
 * Drop-in boundary for the magnification hot path of fbartolic/caustics.  All
 * pointers are caller-owned DEVICE buffers (complex128 = two interleaved
 * doubles), `stream` is a cudaStream_t (NULL = legacy default stream).  Calls
 * launch asynchronously on that stream, never synchronise the device, never
 * allocate and never throw.  The return value is a launch status (CGB_OK or an
 * error code, message in cgb_last_error()); per-item outcomes (convergence,
 * ambiguous image counts, ...) are written as CGB_ST_* bits into the optional
 * `status` buffer (uint32 per item) when the kernels run.
 */
#ifndef CAUSTICS_GB300_H
#define CAUSTICS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CGB_ABI_VERSION 6

/* launch status */
#define CGB_OK 0
#define CGB_ERR_INVALID 1     /* bad argument (null buffer, negative size, bad lens, ...) */
#define CGB_ERR_CUDA 2        /* CUDA launch error */
#define CGB_ERR_UNSUPPORTED 3 /* valid but unsupported request (degree, buffer size) */

/* arithmetic of the root solver / quadrature */
#define CGB_PREC_FP64 0      /* the reference's FP64 Aberth iteration, FP64 quadrature */
#define CGB_PREC_MIXED 1     /* FP32 Aberth + compensated double-float stage + FP64 polish; FP32 LD nodes */
#define CGB_PREC_FP64_COMP 2 /* the reference's compensated FP64 Aberth */

/* per-item status bits */
#define CGB_ST_NOCONV 1u     /* a root solve reached itmax */
#define CGB_ST_AMBIGUOUS 2u  /* a lens-equation residual within x30 of the 1e-6 image threshold */
#define CGB_ST_FALLBACK 4u   /* the mixed solver fell back to FP64 Aberth */
#define CGB_ST_MERGE 8u      /* contour linking left open segments / overflowed */
#define CGB_ST_CAPACITY 16u  /* limb or contour buffers too small (cannot arise at the accepted npts_limb:
                                the contour buffer holds every limb image plus the closing points) */
#define CGB_ST_INVALID 32u   /* non-finite input (source position, coefficient, time, curve parameter) or, in the
                                batched entry points, a curve with s, q or rho not positive or tE zero: the item
                                is not evaluated and its outputs are NaN (the reference returns NaN or garbage
                                for such inputs) */

/* Lens parameters exactly as the reference's keyword arguments:
 * binary (nlenses=2): s, q;  triple (nlenses=3): s, q, q3, r3, psi
 * (src/caustics/point_source.py:1763-1817). */
typedef struct cgb_lens_params {
  int32_t nlenses;
  double s, q;
  double q3, r3, psi;
} cgb_lens_params;

/* Options of mag_extended_source / mag (src/caustics/extended_source.py:741-752,
 * src/caustics/lightcurve.py:99-110). */
typedef struct cgb_es_options {
  int32_t npts_limb;      /* reference defaults: 150 (mag_extended_source), 200 (mag) */
  int32_t limb_darkening; /* 0 = uniform source, 1 = linear limb darkening */
  double u1;              /* linear limb-darkening coefficient */
  int32_t npts_ld;        /* Gauss-Legendre nodes per P/Q integral (2..128), reference default 100 */
  int32_t roots_itmax;    /* reference default 2500 */
  int32_t precision;      /* CGB_PREC_FP64 or CGB_PREC_MIXED */
  int32_t grid;           /* CTAs to launch, 0 = automatic */
  int32_t queue_chunk;    /* batched light curves: work items taken per queue grab (>= 1) */
  int32_t ld_group;       /* lanes sharing one contour point's quadrature nodes: 1, 2, 4 or 8 */
  int32_t labelling;      /* limb image row order: 0 = the reference's warm-start chain, reproduced
                             exactly (faithful FP64 solves on ambiguous steps); 1 = nearest-root
                             matching everywhere (faster; other gaps get refined where the reference
                             would have labelled rows differently: up to 4e-4 measured, 6e-5 on the
                             bench light curve) */
  double grad_fp64_above; /* mixed-precision adjoints: a contour point whose image tangents |dz/dtheta|
                             (own or neighbours', ~1/|det J|) exceed this runs its limb-darkening
                             quadrature in FP64; 0 = default (6), < 0 = every point in FP64 */
  int32_t triple_routing; /* cgb_mag with triple lenses: 0 = contour integral at every point, as the
                             reference's mag() (src/caustics/lightcurve.py:226-227); 1 = the reference's
                             triple hexadecapole (src/caustics/multipole.py:220-229) and the triple branch of its
                             proximity test as written (lightcurve.py:37-46: third-lens terms at -r3, f''
                             term e3/(z+r3)^3), which accepts points where the hexadecapole is tens of percent
                             off; 2 = the same test with the third lens where the lens equation puts it (r3)
                             and f'' = -2 sum eps_j/(z - r_j)^3 */
  int32_t cta_threads;    /* threads per contour-kernel CTA (one CTA per extended-source evaluation):
                             64, 128 or 256; 0 = automatic (128 for the forward at npts_limb <= 256,
                             else 256); fewer threads let more evaluations share an SM where shared
                             memory allows (the phases run on few threads at small npts_limb); a
                             launch-shape knob that changes results only in the summation order */
  int32_t point_lanes;    /* batched light curves, per-point pass (roots, hexadecapole, routing): threads per
                             polynomial, 0 or 1 = one thread per point, 8 = a group of 8 lanes per point
                             (one lane per root, simultaneous Aberth steps; forward only, the adjoint's
                             pass takes one thread per point); roots agree to rounding, so results and
                             routing agree except where a point's test sits on its threshold */
} cgb_es_options;

/* Parameters of one binary-lens light curve for the batched entry points: lens
 * (s, q), source radius and linear limb darkening (rho, u1), and the
 * rectilinear trajectory w(t) = (u0 cos alpha + tau sin alpha)
 * + i (-u0 sin alpha + tau cos alpha), tau = (t - t0) / tE
 * (src/caustics/trajectory.py:152-155 with pi_E = 0). */
typedef struct cgb_curve_params {
  double s, q, rho, u1, u0, alpha, t0, tE;
} cgb_curve_params;

/* One triple-lens light curve: the lens as cgb_lens_params (s, q, q3, r3, psi;
 * masses e1 = q/(1+q+q3), e2 = q e1, third lens at r3 e^{i psi},
 * src/caustics/point_source.py:1807-1817), then the source and the
 * trajectory as cgb_curve_params. */
typedef struct cgb_curve_params_triple {
  double s, q, q3, r3, psi, rho, u1, u0, alpha, t0, tE;
} cgb_curve_params_triple;

/* Message of the last failed call on this thread ("" if none). */
const char *cgb_last_error(void);

/* CGB_ABI_VERSION of the loaded library. */
int32_t cgb_abi_version(void);

/* Gauss-Legendre nodes (ascending) and weights on [-1, 1]; host-only, needs no
 * GPU.  Replaces numpy.polynomial.legendre.leggauss in
 * src/caustics/integrate.py:18-21. */
int cgb_gauss_legendre(int32_t n, double *x, double *w);

/* Roots of n polynomials of degree deg (4, 5, 6 or 10).
 * coeffs: complex128[n, deg+1], low -> high order; roots: complex128[n, deg];
 * roots_init: complex128[n, deg] warm start or NULL (cold start).
 * Replaces the XLA custom calls cpu_ehrlich_aberth / gpu_ehrlich_aberth
 * (lib/ehrlich_aberth/cpu_ops.cc:15-81, kernels.cc.cu:44-112) bound by the
 * ehrlich_aberth primitive (src/caustics/ehrlich_aberth_primitive.py:98-244). */
int cgb_ea_solve(const double *coeffs, const double *roots_init, double *roots, int64_t n, int32_t deg,
                 int32_t itmax, int32_t precision, uint32_t *status, void *stream);

/* Coefficients of the lens-equation polynomial of n source positions w
 * (complex128[n], the centre-of-mass frame of the other entry points; shifted
 * by x_cm = s(1-q)/(2(1+q)) as mag_point_source does): coeffs complex128[n,
 * nlenses^2 + 2], low -> high (the order cgb_ea_solve takes), FP64.  Replaces
 * _poly_coeffs_binary / _poly_coeffs_triple (src/caustics/point_source.py:17-86,
 * 89-1479, highest order first there), computed in product form. */
int cgb_lens_polynomial(const double *w, double *coeffs, int64_t n, cgb_lens_params lens, void *stream);

/* Implicit-function derivatives of the roots returned by cgb_ea_solve, the
 * JVP rule of the reference's primitive (src/caustics/ehrlich_aberth_primitive.py:252-312):
 * dz_r = -sum_k z_r^k dp_k / p'(z_r), coefficients low -> high.
 * jvp: dcoeffs complex128[n, deg+1] -> droots complex128[n, deg].
 * vjp: ct_roots complex128[n, deg] -> ct_coeffs complex128[n, deg+1], the
 * transpose of the JVP map (conjugate = 0, JAX's convention) or its conjugate
 * transpose (conjugate = 1, torch's convention for complex tensors). */
int cgb_ea_roots_jvp(const double *coeffs, const double *roots, const double *dcoeffs, double *droots, int64_t n,
                     int32_t deg, void *stream);
int cgb_ea_roots_vjp(const double *coeffs, const double *roots, const double *ct_roots, double *ct_coeffs, int64_t n,
                     int32_t deg, int32_t conjugate, void *stream);

/* The reference's legacy XLA GPU custom-call signature with its opaque
 * descriptor {int size, deg, itmax; bool compensated}
 * (lib/ehrlich_aberth/kernels.h:11-20, gpu_ops.cc:14-25): buffers[0] = coeffs,
 * buffers[1] = roots.  Errors are reported through cgb_last_error(). */
void gpu_ehrlich_aberth(void *stream, void **buffers, const char *opaque, size_t opaque_len);

/* Source trajectory with annual parallax (replaces
 * AnnualParallaxTrajectory.compute, src/caustics/trajectory.py:106-157,
 * cartesian parametrisation): the projected Sun ephemeris t_jpl, s_e, s_n,
 * s_e_dot, s_n_dot (float64[njpl], t_jpl increasing; the reference builds it with
 * astropy in its constructor) is interpolated linearly, clamped outside its
 * range, at the n times t.  w: complex128[n]; optional dw: complex128[n, 5] =
 * dw / d(u0, t0, tE, piEE, piEN). */
int cgb_parallax_trajectory(const double *t_jpl, const double *s_e, const double *s_n, const double *s_e_dot,
                            const double *s_n_dot, int64_t njpl, const double *t, int64_t n, double u0, double t0,
                            double tE, double piEE, double piEN, double *w, double *dw, void *stream);

/* Log-likelihood of ncurves light curves marginalised over the linear flux
 * parameters (F_s, F_b) with a diagonal inverse covariance (replaces
 * marginalized_log_likelihood(..., dense_covariance=False),
 * src/caustics/linalg.py:10-94; its dense branch does not run in the
 * reference and has no counterpart).  Points offsets[c] .. offsets[c+1]-1
 * (int64, device) of A (magnifications), fobs and C_inv (float64[npoints])
 * belong to curve c.  Outputs: ll float64[ncurves] (the reference returns their
 * sum), optional beta float64[ncurves, 2] = (F_s, F_b), optional dll_dA
 * float64[npoints] = ll_cot[c] * d ll_c / d A_i (ll_cot optional, 1 if null),
 * the cotangent that cgb_mag_lc_batched_vjp takes.  Curves whose normal matrix
 * is singular (fewer than two distinct magnifications) give NaN. */
int cgb_marginalized_log_likelihood(const int64_t *offsets, int64_t ncurves, int64_t npoints, const double *A,
                                    const double *fobs, const double *C_inv, double *beta, double *ll,
                                    double *dll_dA, const double *ll_cot, void *stream);

/* Critical curves and caustics of a binary or triple lens (replaces
 * critical_and_caustic_curves, src/caustics/point_source.py:1582-1649): npts
 * phases on linspace(-pi, pi, npts) (2 <= npts <= 16384), z_cr and z_ca
 * complex128[2 * nlenses, npts], each row one continuous curve (greedy
 * nearest chaining as the reference's match_points), both in the
 * centre-of-mass frame.  status: optional uint32[1] (CGB_ST_NOCONV if a solve
 * reached itmax; the reference's default itmax is 2000).  workspace: device
 * bytes from cgb_critical_curves_workspace_bytes. */
size_t cgb_critical_curves_workspace_bytes(int32_t npts, int32_t nlenses);
int cgb_critical_and_caustic_curves(int32_t npts, cgb_lens_params lens, int32_t itmax, double *z_cr, double *z_ca,
                                    uint32_t *status, void *workspace, size_t workspace_bytes, void *stream);

/* Point-source magnification of n source positions w (complex128[n], in the
 * reference's centre-of-mass frame); mag: float64[n].  Optional outputs:
 * images complex128[n, nlenses^2+1] and image_mask uint32[n] (bit i = image i
 * passes |lens_eq(z) - w| < 1e-6).
 * Replaces mag_point_source (src/caustics/point_source.py:1762-1830). */
int cgb_mag_point_source(const double *w, double *mag, double *images, uint32_t *image_mask, int64_t n,
                         cgb_lens_params lens, int32_t itmax, int32_t precision, uint32_t *status, void *stream);

/* Extended-source magnification by contour integration for n source centres
 * w0 (complex128[n]) of radius rho; mag: float64[n].
 * Replaces mag_extended_source (src/caustics/extended_source.py:741-904). */
int cgb_mag_extended_source(const double *w0, double *mag, int64_t n, double rho, cgb_lens_params lens,
                            const cgb_es_options *opts, uint32_t *status, void *stream);

/* Adjoint of cgb_mag_extended_source: mag float64[n] and, for binary lenses,
 * grad float64[n, 6] = d mag / d(s, q, rho, u1, Re w0, Im w0); for triple
 * lenses grad float64[n, 9] = d mag / d(s, q, rho, u1, Re w0, Im w0, q3, r3, psi)
 * (the reference's parameters, src/caustics/point_source.py:1807-1817) of the discretised
 * contour integral (the limb sampling, segment linking and merging decisions
 * are piecewise constant, as under the reference's autodiff).  The contours are
 * recomputed in the backward pass, not stored.  The reference differentiates
 * mag_extended_source with JAX autodiff through the root primitive's JVP
 * (src/caustics/ehrlich_aberth_primitive.py:254-324). */
int cgb_mag_extended_source_grad(const double *w0, double *mag, double *grad, int64_t n, double rho,
                                 cgb_lens_params lens, const cgb_es_options *opts, uint32_t *status, void *stream);

/* Light curve: hexadecapole where the reference's proximity tests accept it,
 * contour integration elsewhere.  route: uint8[n] output, 1 where the contour
 * integral was used.  Replaces mag (src/caustics/lightcurve.py:99-254). */
int cgb_mag(const double *w, double *mag, uint8_t *route, int64_t n, double rho, cgb_lens_params lens,
            const cgb_es_options *opts, uint32_t *status, void *stream);

/* Workspace (device bytes) of the *_ws forms below for n source positions:
 * one 8-byte first-limb-point row order per position (8 n), 8-byte aligned. */
size_t cgb_mag_extended_source_workspace_bytes(int64_t n);

/* cgb_mag_extended_source, cgb_mag_extended_source_grad and cgb_mag with a
 * caller-owned device workspace of at least
 * cgb_mag_extended_source_workspace_bytes(n) bytes: a separate kernel orders
 * the first limb point of every evaluation ahead of the contour kernel (as the
 * batched entry points do), instead of one lane group per CTA doing it inside
 * the contour kernel.  Same results bit for bit, faster; the workspace is
 * scratch for the duration of the call (stream-ordered).  CGB_ERR_INVALID for
 * a null, short or misaligned workspace when n > 0. */
int cgb_mag_extended_source_ws(const double *w0, double *mag, int64_t n, double rho, cgb_lens_params lens,
                               const cgb_es_options *opts, uint32_t *status, void *workspace,
                               size_t workspace_bytes, void *stream);
int cgb_mag_extended_source_grad_ws(const double *w0, double *mag, double *grad, int64_t n, double rho,
                                    cgb_lens_params lens, const cgb_es_options *opts, uint32_t *status,
                                    void *workspace, size_t workspace_bytes, void *stream);
int cgb_mag_ws(const double *w, double *mag, uint8_t *route, int64_t n, double rho, cgb_lens_params lens,
               const cgb_es_options *opts, uint32_t *status, void *workspace, size_t workspace_bytes, void *stream);

/* Workspace (device bytes) the batched entry points use for npoints points:
 * a 16-byte work-queue header, one 8-byte queue slot per point, then one
 * 8-byte first-limb-point row order per point (16 + 16 npoints).  A workspace
 * of only 16 + 8 npoints bytes is accepted too: the contour kernel then orders
 * each first limb point itself, which is slower. */
size_t cgb_mag_lc_batched_workspace_bytes(int64_t npoints);

/* mag() of ncurves binary-lens light curves of uneven lengths in one pass:
 * points offsets[c] .. offsets[c+1]-1 (int64, device) belong to curve c
 * (curves: cgb_curve_params[ncurves], device) at times t (float64[npoints]).
 * The per-point pass computes the hexadecapole and the routing tests and queues
 * the points that need contour integration; a persistent kernel then drains
 * the device queue.  mag float64[npoints], route uint8[npoints] (1 = contour).
 * Replaces a loop of mag() calls (src/caustics/lightcurve.py:99-254), one per
 * curve. */
int cgb_mag_lc_batched(const int64_t *offsets, const double *t, const cgb_curve_params *curves, int64_t ncurves,
                       int64_t npoints, double *mag, uint8_t *route, uint32_t *status, const cgb_es_options *opts,
                       void *workspace, size_t workspace_bytes, void *stream);

/* cgb_mag_lc_batched for triple-lens light curves (curves:
 * cgb_curve_params_triple[ncurves], device), forward only: as the reference's
 * mag() (src/caustics/lightcurve.py:226-227) every point takes the contour
 * integral (route 1), so opts->triple_routing must be 0 (else
 * CGB_ERR_UNSUPPORTED).  Same workspace as cgb_mag_lc_batched.  Under
 * CGB_PREC_MIXED a curve with a mass fraction below 1e-2 keeps the mixed
 * solver (its roots fall back to FP64 one by one: correct, slower); the
 * single-curve cgb_mag takes FP64 for such lenses from the start, and
 * precision FP64 does the same here. */
int cgb_mag_lc_batched_triple(const int64_t *offsets, const double *t, const cgb_curve_params_triple *curves,
                              int64_t ncurves, int64_t npoints, double *mag, uint8_t *route, uint32_t *status,
                              const cgb_es_options *opts, void *workspace, size_t workspace_bytes, void *stream);

/* cgb_mag_lc_batched without a workspace argument and without allocating: the
 * queue (and, for calls of at most 131,072 points, the first-limb-point row
 * orders) lives in a file-scope device array of the library (2 MiB + 16 B per
 * device), so npoints is limited to 262,144 (larger calls fail with
 * CGB_ERR_UNSUPPORTED).  The first call on a device resolves the array's
 * address in that device's context (cudaGetSymbolAddress); make that first call
 * before any stream capture.  The address is kept per device ordinal for the
 * life of the process: it does not survive a cudaDeviceReset or a primary
 * context reset, after which this entry point must not be called again.
 * `stream` must belong to the current device (a stream of another device is
 * refused with CGB_ERR_INVALID).  All calls on one device share the array: two
 * calls in flight at the same time (other streams or threads) race on it and
 * must be serialised by the caller.  No counterpart in the reference. */
int cgb_mag_lc_batched_noalloc(const int64_t *offsets, const double *t, const cgb_curve_params *curves,
                               int64_t ncurves, int64_t npoints, double *mag, uint8_t *route, uint32_t *status,
                               const cgb_es_options *opts, void *stream);

/* Workspace (device bytes) of cgb_mag_lc_batched_vjp for npoints points: that
 * of cgb_mag_lc_batched (16 + 16 npoints) plus one 64-byte gradient row per
 * point (16 + 80 npoints). */
size_t cgb_mag_lc_batched_vjp_workspace_bytes(int64_t npoints);

/* Vector-Jacobian product of cgb_mag_lc_batched: grad float64[ncurves, 8] =
 * sum over the curve's points of cot[i] * d mag_i / d(s, q, rho, u1, u0,
 * alpha, t0, tE).  Hand-written adjoint: implicit-function rule for the images,
 * forward-mode tangents through the hexadecapole, reverse mode through the
 * contour integral with the contours recomputed.  Also writes mag and route.
 * Every sum runs in a fixed order, so repeated calls give identical bits.
 * workspace: cgb_mag_lc_batched_vjp_workspace_bytes(npoints) device bytes.
 * The reference gets this gradient from JAX autodiff of mag()
 * (src/caustics/lightcurve.py:99-254) through its primitive's JVP
 * (src/caustics/ehrlich_aberth_primitive.py:254-324). */
int cgb_mag_lc_batched_vjp(const int64_t *offsets, const double *t, const cgb_curve_params *curves, int64_t ncurves,
                           int64_t npoints, const double *cot, double *grad, double *mag, uint8_t *route,
                           uint32_t *status, const cgb_es_options *opts, void *workspace, size_t workspace_bytes,
                           void *stream);

/* Workspace (device bytes) of cgb_mag_lc_batched_triple_vjp: that of
 * cgb_mag_lc_batched plus one 88-byte gradient row per point (16 + 104 npoints). */
size_t cgb_mag_lc_batched_triple_vjp_workspace_bytes(int64_t npoints);

/* Vector-Jacobian product of cgb_mag_lc_batched_triple: grad float64[ncurves,
 * 11] = sum over the curve's points of cot[i] * d mag_i / d(s, q, q3, r3, psi,
 * rho, u1, u0, alpha, t0, tE), the curve parameters in their own order; the
 * reference gets the lens part from JAX autodiff through the triple parameter
 * conversion (src/caustics/point_source.py:1807-1817).  As
 * cgb_mag_lc_batched_vjp otherwise (every point through the contour
 * integral; fixed-order sums). */
int cgb_mag_lc_batched_triple_vjp(const int64_t *offsets, const double *t, const cgb_curve_params_triple *curves,
                                  int64_t ncurves, int64_t npoints, const double *cot, double *grad, double *mag,
                                  uint8_t *route, uint32_t *status, const cgb_es_options *opts, void *workspace,
                                  size_t workspace_bytes, void *stream);

/* Diagnostics (no counterpart in the reference): cgb_mag_extended_source that
 * also writes, per point, a record of cgb_debug_record_len(npts_limb) doubles:
 * [L, n_contours, merge flags, (start, count, parity, integral) x 13,
 *  clock cycles of the six phases, faithful-labelling solves of the initial
 *  chain (count + 1000 x iterations, first point included) and of the
 *  refinement (same encoding), theta of the limb points in limb order (room
 *  for the largest limb), clock cycles of the refinement's sub-phases:
 *  interval selection and scan; new-point FP32 stages (FP64: whole solves);
 *  FP64 polish and image filter; per-point labelling; faithful labelling; the
 *  new intervals' lengths, insertion and merge into the ranked intervals; then
 *  of the initial sampling: limb solves; first-point labelling and step maps;
 *  chain repair and row permutation; then FP32-stage iterations summed over
 *  the refinement points, and their number]. */
int cgb_debug_extended_source(const double *w0, double *mag, int64_t n, double rho, cgb_lens_params lens,
                              const cgb_es_options *opts, uint32_t *status, double *dbg, void *stream);
int64_t cgb_debug_record_len(int32_t npts_limb);

#ifdef __cplusplus
}
#endif

#endif /* CAUSTICS_GB300_H */
