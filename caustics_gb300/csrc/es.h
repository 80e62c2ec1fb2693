// Extended-source kernel parameters (shared by the launchers and the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "lens.cuh"

namespace cgb {

constexpr int GL_MAX = 64;  // Gauss-Legendre nodes per half interval

// Per-curve parameters of batched light curves (mirrors cgb_curve_params).
struct CurveDev {
  double s, q, rho, u1, u0, alpha, t0, tE;
};
// a triple-lens light curve: the lens as cgb_lens_params (s, q, q3, r3, psi),
// then the source and trajectory as CurveDev
struct CurveDev3 {
  double s, q, q3, r3, psi, rho, u1, u0, alpha, t0, tE;
};

// The lens / source of the item a CTA is integrating.
struct EsItem {
  Lens L;
  double rho, u1;
  cd w0;          // source centre, shifted by x_cm
  double s, q;    // the user's lens parameters (for the adjoint's chain rule)
  double q3, r3, psi;  // ... and the third lens's (triple lenses)
  int64_t curve;  // batched light curves: curve of the point, else -1
  double tau;     // (t - t0) / tE of the point (batched)
};

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
  // batched light curves (null for a single lens): point i belongs to the curve
  // c with offsets[c] <= i < offsets[c+1]; its source is on the rectilinear
  // trajectory at times[i] (trajectory.py:152-155 with pi_E = 0)
  const CurveDev *curves;
  const CurveDev3 *curves3;  // triple-lens light curves (forward only), instead of curves
  const int64_t *offsets;
  const double *times;
  int64_t ncurves;
  // persistent work queue (null: static round-robin over items)
  unsigned long long *qhead;  // next item to take
  const int64_t *qcount;      // number of queued items
  const int64_t *qlist;       // queued point indices
  int qchunk;                 // items taken per grab
  int ld_group;               // lanes sharing one contour point's quadrature nodes (1, 2, 4, 8)
  int threads;                // threads of a contour-kernel CTA (64, 128 or 256; 0 = chosen at launch)
  int point_lanes;            // per-point pass: threads per polynomial (1, or 8 = a lane group per point)
  double grad_amp2;           // mixed adjoint: FP64 quadrature where max |dz/dtheta|^2 exceeds this
  int nearest;                // 1: nearest-root row labelling (no faithful solves)
  // row order of each item's first limb point, filled by es_first_order_kernel
  // ahead of the contour kernel (indexed by item ordinal); null: the contour
  // kernel orders it itself
  const uint64_t *perm0;
  // adjoint (GRAD kernels): per-point gradient rows [n][6] of
  // (s, q, rho, u1, Re w, Im w) ([n][9] with (q3, r3, psi) for triple lenses),
  // or for batched light curves the cotangent
  // weighted sum per curve [ncurves][8] of (s, q, rho, u1, u0, alpha, t0, tE)
  double *gout;
  const double *cot;
  double *grow;   // batched adjoint: cotangent-weighted gradient row [npoints][8] per point
  double *cgrad;
  double s_user, q_user;  // single-lens parameters (for the adjoint's chain rule)
  double q3_user, r3_user, psi_user;  // triple lenses: the third lens (adjoint chain rule)
  double *dbg;  // optional per-point diagnostics (cgb_debug_extended_source), stride ES_DBG_STRIDE(Lcap)
  double gl_x[2][GL_MAX], gl_w[2][GL_MAX];
};

// diagnostics record: [L, ncont, flags, (start, count, parity, integral) x 13,
// clock64 at the end of phases A..F (6) and the start (1) + 1 spare, theta[0..L)]
#define ES_DBG_CLK (3 + 4 * 13)
#define ES_DBG_HEAD (ES_DBG_CLK + 8)
#define ES_DBG_SUB 9  // refinement and initial-sampling sub-phase clocks
#define ES_DBG_STRIDE(lcap) (ES_DBG_HEAD + (lcap) + ES_DBG_SUB + 2)  // ... stored after theta, then 2 counters

size_t es_smem_bytes(const EsParams &P, int nl, bool grad = false);

// adjoint of the extended-source magnification (binary lenses)
cudaError_t launch_es_grad(const EsParams &P, const double *w0, const uint8_t *route, int64_t n, double *mag,
                           uint32_t *status, int precision, int grid, cudaStream_t stream);

cudaError_t launch_es(const EsParams &P, const double *w0, const int64_t *index, int64_t n, double *mag,
                      uint32_t *status, int precision, int grid, cudaStream_t stream);

// Only the points with route[i] != 0 are integrated; status is OR-ed in.
cudaError_t launch_es_routed(const EsParams &P, const double *w0, const uint8_t *route, int64_t n, double *mag,
                             uint32_t *status, int precision, int grid, cudaStream_t stream);

// Per-point pass of batched light curves; routed points are appended to the
// device queue (qcount, qlist).  grad: hexadecapole-routed points add their
// cotangent-weighted gradient to P.cgrad.
cudaError_t launch_lc_points_batched_triple(const EsParams &P, int64_t n, double *mag, uint8_t *route,
                                            uint32_t *status, unsigned long long *qcount, int64_t *qlist,
                                            cudaStream_t stream, double *grow = nullptr);
cudaError_t launch_lc_points_batched(const EsParams &P, int64_t n, double *mag, uint8_t *route, uint32_t *status,
                                     int precision, unsigned long long *qcount, int64_t *qlist, bool grad,
                                     cudaStream_t stream);

// Per-curve sums of the batched adjoint's point rows: cgrad[c][k] = sum over
// offsets[c] <= i < offsets[c+1] of grow[i][k], in a fixed order (deterministic).
cudaError_t launch_curve_grad_reduce(const int64_t *offsets, int64_t ncurves, const double *grow, double *cgrad,
                                     cudaStream_t stream, int ncols = 8);

// Gauss-Legendre nodes/weights on [-1, 1], ascending (host)
void gauss_legendre(int n, double *x, double *w);

}  // namespace cgb
