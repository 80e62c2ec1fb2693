// C ABI of libcaustics_gb300 (declared in include/caustics_gb300.h).
//
// Every entry point takes caller-owned device buffers and a cudaStream_t,
// launches asynchronously, never synchronises the device, never allocates, and
// returns an int status (0 = launched).  Errors never cross the ABI as C++
// exceptions; the message of the last failure on the calling thread is
// available from cgb_last_error().
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <unordered_map>

#include "../../include/caustics_gb300.h"
#include "es.h"
#include "internal.h"

namespace {

thread_local char g_err[512] = "";

int fail(int code, const char *fmt, const char *detail = "") {
  snprintf(g_err, sizeof(g_err), fmt, detail);
  return code;
}

int cuda_status(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return CGB_OK;
  snprintf(g_err, sizeof(g_err), "%s: %s", what, cudaGetErrorString(e));
  return CGB_ERR_CUDA;
}

bool lens_ok(const cgb_lens_params &p) {
  if (p.nlenses != 2 && p.nlenses != 3) return false;
  if (!(p.s > 0) || !(p.q > 0) || !isfinite(p.s) || !isfinite(p.q)) return false;
  if (p.nlenses == 3 && (!(p.q3 >= 0) || !isfinite(p.r3) || !isfinite(p.psi))) return false;
  return true;
}

Lens lens_of(const cgb_lens_params &p) { return make_lens(p.nlenses, p.s, p.q, p.q3, p.r3, p.psi); }

// Mixed precision needs FP32 to separate the roots.  Around a lens of small
// mass fraction eps, images cluster within ~sqrt(eps) of it, and a degree-10
// polynomial evaluated in FP32 cannot tell them apart: on 1000 random triple
// systems (q ~ logU[1e-4, 1], q3 ~ logU[1e-4, 1e-1]) the mixed solver fell back
// to FP64 for 91-100 % of the sources whenever a mass fraction was below 1e-2,
// and for 17 % above.  Such triple lenses go to the FP64 solver directly;
// binary lenses keep the mixed solver at every mass ratio.
int solver_precision(const cgb_lens_params &p, int precision) {
  if (precision != CGB_PREC_MIXED || p.nlenses != 3) return precision;
  const Lens L = lens_of(p);
  for (int j = 0; j < 3; ++j)
    if (L.eps[j] < 1e-2) return CGB_PREC_FP64;
  return precision;
}

// The point-source kernels solve one polynomial per thread.  For degree 10
// the mixed solver is slower there than FP64 on every triple system measured
// (2^20 positions each: 5.0-11.3M/s against 16.2-18.2M/s, fallback rates 0 to
// 28 %): the FP32 and compensated stages run longer than the FP64 iteration
// they replace.  Triple lenses therefore take the FP64 solver in the
// point-source kernels; the contour kernel keeps solver_precision's choice
// (its mixed path measured 1.0-2.9x faster than FP64 on the same systems).
int point_source_precision(const cgb_lens_params &p, int precision) {
  if (precision == CGB_PREC_MIXED && p.nlenses == 3) return CGB_PREC_FP64;
  return precision;
}

int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

}  // namespace

namespace cgb {

void gauss_legendre(int n, double *x, double *w) {
  // Newton iteration on P_n from the Chebyshev-like first guess, with the
  // three-term recurrence for P_n and P_n' (Golub-Welsch nodes, classic form)
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = cos(pi * (i + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p0 = 0.0;
      for (int k = 0; k < n; ++k) {
        double p2 = p0;
        p0 = p1;
        p1 = ((2.0 * k + 1.0) * z * p0 - k * p2) / (k + 1.0);
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) {
        // one more evaluation of the derivative at the converged node
        p1 = 1.0;
        p0 = 0.0;
        for (int k = 0; k < n; ++k) {
          double p2 = p0;
          p0 = p1;
          p1 = ((2.0 * k + 1.0) * z * p0 - k * p2) / (k + 1.0);
        }
        dp = n * (z * p1 - p0) / (z * z - 1.0);
        break;
      }
    }
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

static int make_es_params(const cgb_lens_params &lens, double rho, const cgb_es_options *o, EsParams &P) {
  if (!o) return fail(CGB_ERR_INVALID, "options pointer is null%s");
  if (!lens_ok(lens)) return fail(CGB_ERR_INVALID, "invalid lens parameters%s");
  if (!(rho > 0) || !isfinite(rho)) return fail(CGB_ERR_INVALID, "rho must be positive and finite%s");
  if (o->npts_limb < 8) return fail(CGB_ERR_INVALID, "npts_limb must be >= 8%s");
  if (o->limb_darkening && (o->npts_ld < 2 || o->npts_ld > 2 * GL_MAX))
    return fail(CGB_ERR_INVALID, "npts_ld must be in [2, 128]%s");
  if (o->precision != CGB_PREC_FP64 && o->precision != CGB_PREC_MIXED)
    return fail(CGB_ERR_INVALID, "extended source precision must be FP64 or MIXED%s");
  memset(&P, 0, sizeof(P));
  P.L = lens_of(lens);
  P.rho = rho;
  P.u1 = o->limb_darkening ? o->u1 : 0.0;
  P.niter = 10;
  P.n0 = (int)(0.5 * o->npts_limb);
  P.n_add = (int)((int)(0.5 * o->npts_limb) / P.niter);
  P.Lcap = P.n0 + P.niter * P.n_add;
  const int deg = lens.nlenses * lens.nlenses + 1;
  P.CPcap = deg * (P.Lcap + 1) + 8;
  P.ld = o->limb_darkening ? 1 : 0;
  P.itmax = o->roots_itmax > 0 ? o->roots_itmax : 2500;
  P.ld_group = (o->ld_group == 2 || o->ld_group == 4 || o->ld_group == 8) ? o->ld_group : 1;
  if (o->cta_threads != 0 && o->cta_threads != 64 && o->cta_threads != 128 && o->cta_threads != 256)
    return fail(CGB_ERR_INVALID, "cta_threads must be 0, 64, 128 or 256%s");
  P.threads = o->cta_threads;  // 0: chosen at launch (launch_es_variant)
  if (o->point_lanes != 0 && o->point_lanes != 1 && o->point_lanes != 8)
    return fail(CGB_ERR_INVALID, "point_lanes must be 0, 1 or 8%s");
  P.point_lanes = o->point_lanes == 8 ? 8 : 1;
  if (o->labelling != 0 && o->labelling != 1) return fail(CGB_ERR_INVALID, "labelling must be 0 or 1%s");
  P.nearest = o->labelling;
  {
    // default 6: on the 256 x 1000-point gradient workload, thresholds 2, 3,
    // 4, 6 and 8 took 637, 494, 425, 355 and 327 ms per 64 curves; the largest
    // per-curve difference to the FP64 VJP over the first 64 curves was 1.4e-5,
    // 4.0e-5, 3.2e-5, 2.6e-5 and 1.1e-4 (over all 256: 1.7e-4 at every threshold,
    // from the forward pass of one curve).  Before FP32 nodes near a limb
    // crossing recomputed 1 - r^2 in FP64, threshold 8 was 8e-4 off.
    const double a = o->grad_fp64_above == 0.0 ? 6.0 : o->grad_fp64_above;
    P.grad_amp2 = a < 0.0 ? -1.0 : a * a;
  }
  P.qchunk = o->queue_chunk > 0 ? o->queue_chunk : 1;
  if (P.ld) {
    P.n1 = o->npts_ld / 2;
    P.n2 = o->npts_ld - P.n1;
    gauss_legendre(P.n1, P.gl_x[0], P.gl_w[0]);
    gauss_legendre(P.n2, P.gl_x[1], P.gl_w[1]);
  }
  if (P.Lcap > 4096) return fail(CGB_ERR_UNSUPPORTED, "npts_limb too large (limb buffer > 4096 points)%s");
  size_t smem = es_smem_bytes(P, lens.nlenses, lens.nlenses == 2);
  int dev = 0, maxsmem = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxsmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (maxsmem > 0 && smem + 4096 > (size_t)maxsmem)
    return fail(CGB_ERR_UNSUPPORTED, "npts_limb too large for shared memory%s");
  return CGB_OK;
}

}  // namespace cgb

using namespace cgb;

extern "C" {

const char *cgb_last_error(void) { return g_err; }

int32_t cgb_abi_version(void) { return CGB_ABI_VERSION; }

int cgb_gauss_legendre(int32_t n, double *x, double *w) {
  if (n < 1 || n > 4096 || !x || !w) return fail(CGB_ERR_INVALID, "invalid Gauss-Legendre request%s");
  gauss_legendre(n, x, w);
  return CGB_OK;
}

int cgb_ea_solve(const double *coeffs, const double *roots_init, double *roots, int64_t n, int32_t deg,
                 int32_t itmax, int32_t precision, uint32_t *status, void *stream) {
  if (n < 0) return fail(CGB_ERR_INVALID, "n must be >= 0%s");
  if (n > 0 && (!coeffs || !roots)) return fail(CGB_ERR_INVALID, "null buffer%s");
  if (deg != 4 && deg != 5 && deg != 6 && deg != 10)
    return fail(CGB_ERR_UNSUPPORTED, "degree must be 4, 5, 6 or 10%s");
  if (precision < 0 || precision > 2) return fail(CGB_ERR_INVALID, "unknown precision%s");
  if (itmax < 1) return fail(CGB_ERR_INVALID, "itmax must be >= 1%s");
  return cuda_status(launch_ea_solve(coeffs, roots_init, roots, n, deg, itmax, precision, status,
                                     (cudaStream_t)stream),
                     "cgb_ea_solve launch");
}

int cgb_lens_polynomial(const double *w, double *coeffs, int64_t n, cgb_lens_params lens, void *stream) {
  if (n < 0) return fail(CGB_ERR_INVALID, "n must be >= 0%s");
  if (n > 0 && (!w || !coeffs)) return fail(CGB_ERR_INVALID, "null buffer%s");
  if (!lens_ok(lens)) return fail(CGB_ERR_INVALID, "invalid lens parameters%s");
  return cuda_status(launch_lens_poly(lens_of(lens), w, coeffs, n, (cudaStream_t)stream), "cgb_lens_polynomial launch");
}

int cgb_ea_roots_jvp(const double *coeffs, const double *roots, const double *dcoeffs, double *droots, int64_t n,
                     int32_t deg, void *stream) {
  if (n < 0) return fail(CGB_ERR_INVALID, "n must be >= 0%s");
  if (deg < 1 || deg > 64) return fail(CGB_ERR_INVALID, "degree must be in 1..64%s");
  if (n == 0) return CGB_OK;
  if (!coeffs || !roots || !dcoeffs || !droots) return fail(CGB_ERR_INVALID, "null buffer%s");
  return cuda_status(launch_roots_jvp(coeffs, roots, dcoeffs, droots, n, deg, (cudaStream_t)stream),
                     "cgb_ea_roots_jvp launch");
}

int cgb_ea_roots_vjp(const double *coeffs, const double *roots, const double *ct_roots, double *ct_coeffs, int64_t n,
                     int32_t deg, int32_t conjugate, void *stream) {
  if (n < 0) return fail(CGB_ERR_INVALID, "n must be >= 0%s");
  if (deg < 1 || deg > 64) return fail(CGB_ERR_INVALID, "degree must be in 1..64%s");
  if (n == 0) return CGB_OK;
  if (!coeffs || !roots || !ct_roots || !ct_coeffs) return fail(CGB_ERR_INVALID, "null buffer%s");
  return cuda_status(launch_roots_vjp(coeffs, roots, ct_roots, ct_coeffs, n, deg, conjugate != 0,
                                      (cudaStream_t)stream),
                     "cgb_ea_roots_vjp launch");
}

// The reference's XLA GPU custom call: buffers[0] coeffs complex128[size, deg+1]
// (low -> high), buffers[1] roots complex128[size*deg]; opaque is the packed
// {int size, deg, itmax; bool compensated} descriptor (lib/ehrlich_aberth/kernels.h:11-17).
void gpu_ehrlich_aberth(void *stream, void **buffers, const char *opaque, size_t opaque_len) {
  struct Descriptor {
    int size, deg, itmax;
    bool compensated;
  } d;
  if (opaque_len != sizeof(Descriptor) || !buffers) {
    fail(CGB_ERR_INVALID, "gpu_ehrlich_aberth: invalid opaque descriptor size%s");
    return;
  }
  memcpy(&d, opaque, sizeof(d));
  cgb_ea_solve((const double *)buffers[0], nullptr, (double *)buffers[1], d.size, d.deg, d.itmax,
               d.compensated ? CGB_PREC_FP64_COMP : CGB_PREC_FP64, nullptr, stream);
}

int cgb_parallax_trajectory(const double *t_jpl, const double *s_e, const double *s_n, const double *s_e_dot,
                            const double *s_n_dot, int64_t njpl, const double *t, int64_t n, double u0, double t0,
                            double tE, double piEE, double piEN, double *w, double *dw, void *stream) {
  if (n < 0 || njpl < 1) return fail(CGB_ERR_INVALID, "need n >= 0 and an ephemeris of >= 1 sample%s");
  if (n == 0) return CGB_OK;
  if (!t_jpl || !s_e || !s_n || !s_e_dot || !s_n_dot || !t || !w) return fail(CGB_ERR_INVALID, "null buffer%s");
  if (!(tE > 0) || !isfinite(tE) || !isfinite(u0) || !isfinite(t0) || !isfinite(piEE) || !isfinite(piEN))
    return fail(CGB_ERR_INVALID, "invalid trajectory parameters%s");
  return cuda_status(launch_parallax(t_jpl, s_e, s_n, s_e_dot, s_n_dot, njpl, t, n, u0, t0, tE, piEE, piEN, w, dw,
                                     (cudaStream_t)stream),
                     "cgb_parallax_trajectory launch");
}

int cgb_marginalized_log_likelihood(const int64_t *offsets, int64_t ncurves, int64_t npoints, const double *A,
                                    const double *fobs, const double *C_inv, double *beta, double *ll,
                                    double *dll_dA, const double *ll_cot, void *stream) {
  if (ncurves < 0 || npoints < 0) return fail(CGB_ERR_INVALID, "ncurves and npoints must be >= 0%s");
  if (ncurves == 0) return CGB_OK;
  if (!offsets || !ll || (npoints > 0 && (!A || !fobs || !C_inv))) return fail(CGB_ERR_INVALID, "null buffer%s");
  return cuda_status(launch_marg_ll(offsets, ncurves, A, fobs, C_inv, beta, ll, dll_dA, ll_cot, (cudaStream_t)stream),
                     "cgb_marginalized_log_likelihood launch");
}

size_t cgb_critical_curves_workspace_bytes(int32_t npts, int32_t nlenses) {
  return critical_workspace_bytes(npts, nlenses == 3 ? 3 : 2);
}

int cgb_critical_and_caustic_curves(int32_t npts, cgb_lens_params lens, int32_t itmax, double *z_cr, double *z_ca,
                                    uint32_t *status, void *workspace, size_t workspace_bytes, void *stream) {
  if (npts < 2 || npts > 16384) return fail(CGB_ERR_INVALID, "npts must be in [2, 16384]%s");
  if (!lens_ok(lens)) return fail(CGB_ERR_INVALID, "invalid lens parameters%s");
  if (itmax < 1) return fail(CGB_ERR_INVALID, "itmax must be >= 1%s");
  if (!z_cr || !z_ca) return fail(CGB_ERR_INVALID, "null buffer%s");
  if (!workspace || workspace_bytes < critical_workspace_bytes(npts, lens.nlenses))
    return fail(CGB_ERR_INVALID, "workspace too small (see cgb_critical_curves_workspace_bytes)%s");
  if (status) {
    int rc = cuda_status(cudaMemsetAsync(status, 0, sizeof(uint32_t), (cudaStream_t)stream), "status reset");
    if (rc) return rc;
  }
  return cuda_status(launch_critical(lens_of(lens), npts, itmax, z_cr, z_ca, status, workspace, (cudaStream_t)stream),
                     "cgb_critical_and_caustic_curves launch");
}

int cgb_mag_point_source(const double *w, double *mag, double *images, uint32_t *image_mask, int64_t n,
                         cgb_lens_params lens, int32_t itmax, int32_t precision, uint32_t *status, void *stream) {
  if (n < 0) return fail(CGB_ERR_INVALID, "n must be >= 0%s");
  if (n > 0 && (!w || !mag)) return fail(CGB_ERR_INVALID, "null buffer%s");
  if (!lens_ok(lens)) return fail(CGB_ERR_INVALID, "invalid lens parameters%s");
  if (precision < 0 || precision > 2) return fail(CGB_ERR_INVALID, "unknown precision%s");
  if (itmax < 1) return fail(CGB_ERR_INVALID, "itmax must be >= 1%s");
  return cuda_status(launch_mag_ps(lens_of(lens), w, mag, images, image_mask, n, itmax,
                                   point_source_precision(lens, precision), status,
                                   (cudaStream_t)stream),
                     "cgb_mag_point_source launch");
}

// Workspace of the single-evaluation entry points (the *_ws forms): one
// first-limb-point row order (8 bytes, 8-byte aligned) per source position, so
// that es_first_order_kernel orders every item's first limb point ahead of the
// contour kernel, as in the batched path.
size_t cgb_mag_extended_source_workspace_bytes(int64_t n) { return n > 0 ? 8 * (size_t)n : 0; }

static int es_workspace(EsParams &P, int64_t n, void *ws, size_t ws_bytes) {
  if (n <= 0) return 0;
  if (!ws || ws_bytes < cgb_mag_extended_source_workspace_bytes(n) || ((uintptr_t)ws & 7u))
    return fail(CGB_ERR_INVALID, "workspace: 8 bytes per source position, 8-byte aligned%s");
  P.perm0 = reinterpret_cast<const uint64_t *>(ws);
  return 0;
}

static int mag_extended_source_impl(const double *w0, double *mag, int64_t n, double rho, cgb_lens_params lens,
                                    const cgb_es_options *opts, uint32_t *status, void *ws, size_t ws_bytes,
                                    void *stream) {
  if (n < 0) return fail(CGB_ERR_INVALID, "n must be >= 0%s");
  if (n > 0 && (!w0 || !mag)) return fail(CGB_ERR_INVALID, "null buffer%s");
  EsParams P;
  int rc = make_es_params(lens, rho, opts, P);
  if (rc) return rc;
  if (ws && (rc = es_workspace(P, n, ws, ws_bytes))) return rc;
  int grid = opts->grid > 0 ? opts->grid : (int)((n < 8 * sm_count()) ? n : 8 * sm_count());
  if (grid < 1) grid = 1;
  return cuda_status(launch_es(P, w0, nullptr, n, mag, status, solver_precision(lens, opts->precision), grid,
                               (cudaStream_t)stream),
                     "cgb_mag_extended_source launch");
}

int cgb_mag_extended_source(const double *w0, double *mag, int64_t n, double rho, cgb_lens_params lens,
                            const cgb_es_options *opts, uint32_t *status, void *stream) {
  return mag_extended_source_impl(w0, mag, n, rho, lens, opts, status, nullptr, 0, stream);
}

int cgb_mag_extended_source_ws(const double *w0, double *mag, int64_t n, double rho, cgb_lens_params lens,
                               const cgb_es_options *opts, uint32_t *status, void *workspace,
                               size_t workspace_bytes, void *stream) {
  if (n > 0 && !workspace) return fail(CGB_ERR_INVALID, "null workspace%s");
  return mag_extended_source_impl(w0, mag, n, rho, lens, opts, status, workspace, workspace_bytes, stream);
}

static int mag_extended_source_grad_impl(const double *w0, double *mag, double *grad, int64_t n, double rho,
                                         cgb_lens_params lens, const cgb_es_options *opts, uint32_t *status,
                                         void *ws, size_t ws_bytes, void *stream) {
  if (n < 0 || (n > 0 && (!w0 || !mag || !grad))) return fail(CGB_ERR_INVALID, "invalid buffers%s");
  EsParams P;
  int rc = make_es_params(lens, rho, opts, P);
  if (rc) return rc;
  if (ws && (rc = es_workspace(P, n, ws, ws_bytes))) return rc;
  if (lens.nlenses == 3) {  // the adjoint's accumulators may need shared memory beyond the forward's
    int dev = 0, maxsmem = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maxsmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (maxsmem > 0 && es_smem_bytes(P, 3, true) + 4096 > (size_t)maxsmem)
      return fail(CGB_ERR_UNSUPPORTED, "npts_limb too large for the triple-lens adjoint's shared memory%s");
  }
  P.gout = grad;
  P.s_user = lens.s;
  P.q_user = lens.q;
  P.q3_user = lens.q3;
  P.r3_user = lens.r3;
  P.psi_user = lens.psi;
  int grid = opts->grid > 0 ? opts->grid : (int)((n < 4 * sm_count()) ? n : 4 * sm_count());
  if (grid < 1) grid = 1;
  return cuda_status(launch_es_grad(P, w0, nullptr, n, mag, status, opts->precision, grid, (cudaStream_t)stream),
                     "cgb_mag_extended_source_grad launch");
}

int cgb_mag_extended_source_grad(const double *w0, double *mag, double *grad, int64_t n, double rho,
                                 cgb_lens_params lens, const cgb_es_options *opts, uint32_t *status, void *stream) {
  return mag_extended_source_grad_impl(w0, mag, grad, n, rho, lens, opts, status, nullptr, 0, stream);
}

int cgb_mag_extended_source_grad_ws(const double *w0, double *mag, double *grad, int64_t n, double rho,
                                    cgb_lens_params lens, const cgb_es_options *opts, uint32_t *status,
                                    void *workspace, size_t workspace_bytes, void *stream) {
  if (n > 0 && !workspace) return fail(CGB_ERR_INVALID, "null workspace%s");
  return mag_extended_source_grad_impl(w0, mag, grad, n, rho, lens, opts, status, workspace, workspace_bytes,
                                       stream);
}

// Workspace of the batched entry points: a 16-byte queue header, one queue
// slot per point, then one first-limb-point row order per point.  Only the
// first two are required: with a workspace of 16 + 8 npoints bytes the contour
// kernel orders each first limb point itself (one lane group per block, slower).
size_t cgb_mag_lc_batched_workspace_bytes(int64_t npoints) {
  return 16 + 16 * (size_t)(npoints > 0 ? npoints : 0);
}
static size_t batched_queue_bytes(int64_t npoints) { return 16 + 8 * (size_t)(npoints > 0 ? npoints : 0); }
// The adjoint also keeps one cotangent-weighted gradient row (8 doubles) per
// point, summed per curve in a fixed order afterwards.
size_t cgb_mag_lc_batched_vjp_workspace_bytes(int64_t npoints) {
  return cgb_mag_lc_batched_workspace_bytes(npoints) + 64 * (size_t)(npoints > 0 ? npoints : 0);
}

size_t cgb_mag_lc_batched_triple_vjp_workspace_bytes(int64_t npoints) {
  return cgb_mag_lc_batched_workspace_bytes(npoints) + 88 * (size_t)(npoints > 0 ? npoints : 0);
}

// nl: 2 (curves: cgb_curve_params) or 3 (cgb_curve_params_triple); the
// options are checked against a lens of that many masses (shared memory).
static int batched_setup(const int64_t *offsets, const double *t, const void *curves, int64_t ncurves,
                         int64_t npoints, const cgb_es_options *opts, void *ws, size_t ws_bytes, EsParams &P,
                         int nl = 2) {
  if (ncurves < 1 || npoints < 0) return fail(CGB_ERR_INVALID, "need ncurves >= 1 and npoints >= 0%s");
  if (!offsets || !curves || (npoints > 0 && !t)) return fail(CGB_ERR_INVALID, "null buffer%s");
  if (!ws || ws_bytes < batched_queue_bytes(npoints))
    return fail(CGB_ERR_INVALID, "workspace too small (see cgb_mag_lc_batched_workspace_bytes)%s");
  const cgb_lens_params dummy = nl == 3 ? cgb_lens_params{3, 1.0, 0.5, 0.1, 1.0, 0.0}
                                        : cgb_lens_params{2, 1.0, 1.0, 0.0, 0.0, 0.0};
  int rc = make_es_params(dummy, 1.0, opts, P);
  if (rc) return rc;
  if (nl == 3)
    P.curves3 = reinterpret_cast<const CurveDev3 *>(curves);
  else
    P.curves = reinterpret_cast<const CurveDev *>(curves);
  P.offsets = offsets;
  P.times = t;
  P.ncurves = ncurves;
  P.qcount = reinterpret_cast<const int64_t *>(ws);
  P.qhead = reinterpret_cast<unsigned long long *>((char *)ws + 8);
  P.qlist = reinterpret_cast<const int64_t *>((char *)ws + 16);
  if (ws_bytes >= cgb_mag_lc_batched_workspace_bytes(npoints))
    P.perm0 = reinterpret_cast<const uint64_t *>((char *)ws + batched_queue_bytes(npoints));
  P.qchunk = opts->queue_chunk > 0 ? opts->queue_chunk : 1;
  return CGB_OK;
}

int cgb_mag_lc_batched(const int64_t *offsets, const double *t, const cgb_curve_params *curves, int64_t ncurves,
                       int64_t npoints, double *mag, uint8_t *route, uint32_t *status, const cgb_es_options *opts,
                       void *workspace, size_t workspace_bytes, void *stream) {
  if (npoints > 0 && (!mag || !route)) return fail(CGB_ERR_INVALID, "null buffer%s");
  EsParams P;
  int rc = batched_setup(offsets, t, curves, ncurves, npoints, opts, workspace, workspace_bytes, P);
  if (rc) return rc;
  if (npoints == 0) return CGB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  rc = cuda_status(cudaMemsetAsync(workspace, 0, 16, s), "queue reset");
  if (rc) return rc;
  const int prec_ps = opts->precision == CGB_PREC_MIXED ? MIXED : FP64;
  rc = cuda_status(launch_lc_points_batched(P, npoints, mag, route, status, prec_ps,
                                            (unsigned long long *)workspace, (int64_t *)((char *)workspace + 16), false,
                                            s),
                   "cgb_mag_lc_batched point pass");
  if (rc) return rc;
  return cuda_status(launch_es_routed(P, nullptr, route, npoints, mag, status, opts->precision, opts->grid, s),
                     "cgb_mag_lc_batched contour pass");
}

int cgb_mag_lc_batched_triple(const int64_t *offsets, const double *t, const cgb_curve_params_triple *curves,
                              int64_t ncurves, int64_t npoints, double *mag, uint8_t *route, uint32_t *status,
                              const cgb_es_options *opts, void *workspace, size_t workspace_bytes, void *stream) {
  if (npoints > 0 && (!mag || !route)) return fail(CGB_ERR_INVALID, "null buffer%s");
  if (opts && opts->triple_routing != 0)
    return fail(CGB_ERR_UNSUPPORTED, "batched triple-lens light curves take triple_routing 0%s");
  EsParams P;
  int rc = batched_setup(offsets, t, curves, ncurves, npoints, opts, workspace, workspace_bytes, P, 3);
  if (rc) return rc;
  if (npoints == 0) return CGB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  rc = cuda_status(cudaMemsetAsync(workspace, 0, 16, s), "queue reset");
  if (rc) return rc;
  rc = cuda_status(launch_lc_points_batched_triple(P, npoints, mag, route, status, (unsigned long long *)workspace,
                                                   (int64_t *)((char *)workspace + 16), s),
                   "cgb_mag_lc_batched_triple point pass");
  if (rc) return rc;
  return cuda_status(launch_es_routed(P, nullptr, route, npoints, mag, status, opts->precision, opts->grid, s),
                     "cgb_mag_lc_batched_triple contour pass");
}

int cgb_mag_lc_batched_vjp(const int64_t *offsets, const double *t, const cgb_curve_params *curves, int64_t ncurves,
                           int64_t npoints, const double *cot, double *grad, double *mag, uint8_t *route,
                           uint32_t *status, const cgb_es_options *opts, void *workspace, size_t workspace_bytes,
                           void *stream) {
  if (!grad || (npoints > 0 && (!mag || !route || !cot))) return fail(CGB_ERR_INVALID, "null buffer%s");
  if (!workspace || workspace_bytes < cgb_mag_lc_batched_vjp_workspace_bytes(npoints))
    return fail(CGB_ERR_INVALID, "workspace too small (see cgb_mag_lc_batched_vjp_workspace_bytes)%s");
  EsParams P;
  int rc = batched_setup(offsets, t, curves, ncurves, npoints, opts, workspace, workspace_bytes, P);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  if (npoints == 0)
    return cuda_status(cudaMemsetAsync(grad, 0, sizeof(double) * 8 * (size_t)ncurves, s), "gradient reset");
  rc = cuda_status(cudaMemsetAsync(workspace, 0, 16, s), "queue reset");
  if (rc) return rc;
  P.cot = cot;
  P.cgrad = grad;
  P.grow = reinterpret_cast<double *>((char *)workspace + cgb_mag_lc_batched_workspace_bytes(npoints));
  const int prec_ps = opts->precision == CGB_PREC_MIXED ? MIXED : FP64;
  rc = cuda_status(launch_lc_points_batched(P, npoints, mag, route, status, prec_ps,
                                            (unsigned long long *)workspace, (int64_t *)((char *)workspace + 16), true,
                                            s),
                   "cgb_mag_lc_batched_vjp point pass");
  if (rc) return rc;
  rc = cuda_status(launch_es_grad(P, nullptr, route, npoints, mag, status, opts->precision, opts->grid, s),
                   "cgb_mag_lc_batched_vjp contour pass");
  if (rc) return rc;
  return cuda_status(launch_curve_grad_reduce(offsets, ncurves, P.grow, grad, s), "cgb_mag_lc_batched_vjp curve sums");
}

int cgb_mag_lc_batched_triple_vjp(const int64_t *offsets, const double *t, const cgb_curve_params_triple *curves,
                                  int64_t ncurves, int64_t npoints, const double *cot, double *grad, double *mag,
                                  uint8_t *route, uint32_t *status, const cgb_es_options *opts, void *workspace,
                                  size_t workspace_bytes, void *stream) {
  if (!grad || (npoints > 0 && (!mag || !route || !cot))) return fail(CGB_ERR_INVALID, "null buffer%s");
  if (opts && opts->triple_routing != 0)
    return fail(CGB_ERR_UNSUPPORTED, "batched triple-lens light curves take triple_routing 0%s");
  if (!workspace || workspace_bytes < cgb_mag_lc_batched_triple_vjp_workspace_bytes(npoints))
    return fail(CGB_ERR_INVALID, "workspace too small (see cgb_mag_lc_batched_triple_vjp_workspace_bytes)%s");
  EsParams P;
  int rc = batched_setup(offsets, t, curves, ncurves, npoints, opts, workspace, workspace_bytes, P, 3);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  if (npoints == 0)
    return cuda_status(cudaMemsetAsync(grad, 0, sizeof(double) * 11 * (size_t)ncurves, s), "gradient reset");
  {  // the adjoint kernel's shared memory for a triple lens
    size_t smem = es_smem_bytes(P, 3, true);
    int dev = 0, maxsmem = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maxsmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (maxsmem > 0 && smem + 4096 > (size_t)maxsmem)
      return fail(CGB_ERR_UNSUPPORTED, "npts_limb too large for the triple-lens adjoint's shared memory%s");
  }
  rc = cuda_status(cudaMemsetAsync(workspace, 0, 16, s), "queue reset");
  if (rc) return rc;
  P.cot = cot;
  P.cgrad = grad;
  P.grow = reinterpret_cast<double *>((char *)workspace + cgb_mag_lc_batched_workspace_bytes(npoints));
  rc = cuda_status(launch_lc_points_batched_triple(P, npoints, mag, route, status, (unsigned long long *)workspace,
                                                   (int64_t *)((char *)workspace + 16), s, P.grow),
                   "cgb_mag_lc_batched_triple_vjp point pass");
  if (rc) return rc;
  rc = cuda_status(launch_es_grad(P, nullptr, route, npoints, mag, status, opts->precision, opts->grid, s),
                   "cgb_mag_lc_batched_triple_vjp contour pass");
  if (rc) return rc;
  return cuda_status(launch_curve_grad_reduce(offsets, ncurves, P.grow, grad, s, 11),
                     "cgb_mag_lc_batched_triple_vjp curve sums");
}

int cgb_debug_extended_source(const double *w0, double *mag, int64_t n, double rho, cgb_lens_params lens,
                              const cgb_es_options *opts, uint32_t *status, double *dbg, void *stream) {
  if (n < 0 || (n > 0 && (!w0 || !mag || !dbg))) return fail(CGB_ERR_INVALID, "invalid buffers%s");
  EsParams P;
  int rc = make_es_params(lens, rho, opts, P);
  if (rc) return rc;
  P.dbg = dbg;
  int grid = opts->grid > 0 ? opts->grid : (int)((n < 8 * sm_count()) ? n : 8 * sm_count());
  if (grid < 1) grid = 1;
  return cuda_status(launch_es(P, w0, nullptr, n, mag, status, opts->precision, grid, (cudaStream_t)stream),
                     "cgb_debug_extended_source launch");
}

int64_t cgb_debug_record_len(int32_t npts_limb) {
  int n0 = (int)(0.5 * npts_limb);
  return ES_DBG_STRIDE(n0 + 10 * (n0 / 10));
}

static int mag_impl(const double *w, double *mag, uint8_t *route, int64_t n, double rho, cgb_lens_params lens,
                    const cgb_es_options *opts, uint32_t *status, void *ws, size_t ws_bytes, void *stream) {
  if (n < 0) return fail(CGB_ERR_INVALID, "n must be >= 0%s");
  if (n > 0 && (!w || !mag || !route)) return fail(CGB_ERR_INVALID, "null buffer%s");
  EsParams P;
  int rc = make_es_params(lens, rho, opts, P);
  if (rc) return rc;
  if (ws && (rc = es_workspace(P, n, ws, ws_bytes))) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const int prec = solver_precision(lens, opts->precision);
  const int prec_ps = point_source_precision(lens, prec) == CGB_PREC_MIXED ? MIXED : FP64;
  if (opts->triple_routing < 0 || opts->triple_routing > 2)
    return fail(CGB_ERR_INVALID, "triple_routing must be 0, 1 or 2%s");
  rc = cuda_status(launch_lc_points(P.L, lens.q, w, rho, mag, route, n, P.itmax, prec_ps, status,
                                    opts->triple_routing, s),
                   "cgb_mag point pass launch");
  if (rc) return rc;
  int grid = opts->grid > 0 ? opts->grid : (int)((n < 8 * sm_count()) ? n : 8 * sm_count());
  if (grid < 1) grid = 1;
  return cuda_status(launch_es_routed(P, w, route, n, mag, status, prec, grid, s),
                     "cgb_mag contour pass launch");
}

int cgb_mag(const double *w, double *mag, uint8_t *route, int64_t n, double rho, cgb_lens_params lens,
            const cgb_es_options *opts, uint32_t *status, void *stream) {
  return mag_impl(w, mag, route, n, rho, lens, opts, status, nullptr, 0, stream);
}

int cgb_mag_ws(const double *w, double *mag, uint8_t *route, int64_t n, double rho, cgb_lens_params lens,
               const cgb_es_options *opts, uint32_t *status, void *workspace, size_t workspace_bytes, void *stream) {
  if (n > 0 && !workspace) return fail(CGB_ERR_INVALID, "null workspace%s");
  return mag_impl(w, mag, route, n, rho, lens, opts, status, workspace, workspace_bytes, stream);
}

// ---- batched light curves without any allocation ----
// Some callers cannot hand over a workspace and must not allocate device memory
// themselves: an XLA custom-call handler gets every buffer from XLA's own
// buffer assignment (the reference's GPU kernel called cudaMalloc per call
// instead, lib/ehrlich_aberth/kernels.cc.cu:72-76), and a plain C caller that
// binds only this ABI may run where no allocator is at hand.  For them the
// queue header and queue slots live in a fixed, file-scope device array (and
// the first-point row orders too, for calls of at most 131,072 points).
namespace {
constexpr int64_t kNoAllocMaxPoints = 1 << 18;  // 262,144 light-curve points per call
constexpr size_t kNoAllocScratchBytes = 16 + 8 * (size_t)kNoAllocMaxPoints;  // 2 MiB + 16 B per device
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
constexpr int kNoAllocMaxDevices = 64;
void *g_noalloc_ptr[kNoAllocMaxDevices];  // device address of the scratch, per device ordinal
std::mutex g_noalloc_mu;
}  // namespace

extern "C" int cgb_mag_lc_batched_noalloc(const int64_t *offsets, const double *t, const cgb_curve_params *curves,
                                          int64_t ncurves, int64_t npoints, double *mag, uint8_t *route,
                                          uint32_t *status, const cgb_es_options *opts, void *stream) {
  if (npoints > kNoAllocMaxPoints)
    return fail(CGB_ERR_UNSUPPORTED,
                "cgb_mag_lc_batched_noalloc: npoints exceeds the static scratch (262144 points)%s");
  int dev = -1;
  int rc = cuda_status(cudaGetDevice(&dev), "cgb_mag_lc_batched_noalloc: current device");
  if (rc) return rc;
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return fail(CGB_ERR_UNSUPPORTED, "cgb_mag_lc_batched_noalloc: device ordinal out of range%s");
  if (stream) {  // the scratch is the current device's: the stream must be on it too
    int sdev = -1;
    rc = cuda_status(cudaStreamGetDevice((cudaStream_t)stream, &sdev), "cgb_mag_lc_batched_noalloc: stream device");
    if (rc) return rc;
    if (sdev != dev)
      return fail(CGB_ERR_INVALID,
                  "cgb_mag_lc_batched_noalloc: the stream belongs to another device than the current one%s");
  }
  void *ws = nullptr;
  {
    // first call on a device: resolve the array's address in that device's context
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void *p = nullptr;
      rc = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cgb_mag_lc_batched_noalloc: scratch address");
      if (rc) return rc;
      g_noalloc_ptr[dev] = p;
    }
    ws = g_noalloc_ptr[dev];
  }
  // the call zeroes the 16-byte queue header on `stream`; the slots need no reset
  return cgb_mag_lc_batched(offsets, t, curves, ncurves, npoints, mag, route, status, opts, ws, kNoAllocScratchBytes,
                            stream);
}

}  // extern "C"
