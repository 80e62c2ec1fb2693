/*
 * ORACLE — test infrastructure only.  CPU restatement (plain C, FP64) of the
 * Ehrlich-Aberth simultaneous root solver of fbartolic/caustics.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library;
 * the product path never does.
 *
 * Follows, step by step:
 *   lib/ehrlich_aberth/ehrlich_aberth.h:27-58   Aberth correction (forward / reversed)
 *   lib/ehrlich_aberth/ehrlich_aberth.h:60-150  plain iteration, stopping test |p(z)| <= EPS*b
 *   lib/ehrlich_aberth/ehrlich_aberth.h:153-292 compensated second stage
 *   lib/ehrlich_aberth/horner.h:30-35,44-84     gamma constant, TwoSum, TwoProd (FMA), complex EFTs
 *   lib/ehrlich_aberth/horner.h:164-208         Priest doubly-compensated summation of 4 terms
 *   lib/ehrlich_aberth/horner.h:219-267,281-385 real / complex / compensated Horner (and reversed)
 *   lib/ehrlich_aberth/init_est.h:37-102        initial estimates from the upper convex hull
 *
 * Coefficients are complex128, low -> high order (poly[0] + poly[1] z + ...),
 * as the reference's custom call receives them.
 *
 * init_mode: 0 = complex initial guesses r*exp(i*phi) (what the product uses);
 *            1 = the reference's real-valued guesses r*sin(phi) (init_est.h:95
 *                applies the comma operator), for bit-level comparison with it.
 * Returns per polynomial the number of outer iterations used, or -1 when itmax
 * was reached without convergence (the reference prints and asserts there).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

typedef struct { double re, im; } cplx;

static const double EPS = DBL_EPSILON / 2;

static inline cplx cmk(double re, double im) { cplx c = {re, im}; return c; }
static inline cplx cadd(cplx a, cplx b) { return cmk(a.re + b.re, a.im + b.im); }
static inline cplx csub(cplx a, cplx b) { return cmk(a.re - b.re, a.im - b.im); }
static inline cplx cmul(cplx a, cplx b) { return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cplx cscale(cplx a, double s) { return cmk(a.re * s, a.im * s); }
static inline double cabs_(cplx a) { return hypot(a.re, a.im); }
/* Smith's algorithm for a / b. */
static inline cplx cdiv(cplx a, cplx b) {
  if (fabs(b.re) >= fabs(b.im)) {
    double r = b.im / b.re, d = b.re + b.im * r;
    return cmk((a.re + a.im * r) / d, (a.im - a.re * r) / d);
  } else {
    double r = b.re / b.im, d = b.re * r + b.im;
    return cmk((a.re * r + a.im) / d, (a.im * r - a.re) / d);
  }
}
static inline cplx crecip(cplx b) { return cdiv(cmk(1.0, 0.0), b); }

/* ---- error-free transforms (horner.h:37-84) ---- */
static inline void two_sum(double a, double b, double *s, double *e) {
  *s = a + b;
  double t = *s - a;
  *e = (a - (*s - t)) + (b - t);
}
static inline void two_prod(double a, double b, double *p, double *e) {
  *p = a * b;
  *e = fma(a, b, -*p);
}
/* product a*b = res + e1 + e2 + e3 exactly (complex). */
static inline void two_prod_c(cplx a, cplx b, cplx *res, cplx *e1, cplx *e2, cplx *e3) {
  double p0, q0, p1, q1, p2, q2, p3, q3, s4, r4, s5, r5;
  two_prod(a.re, b.re, &p0, &q0);
  two_prod(a.im, b.im, &p1, &q1);
  two_prod(a.re, b.im, &p2, &q2);
  two_prod(a.im, b.re, &p3, &q3);
  two_sum(p0, -p1, &s4, &r4);
  two_sum(p2, p3, &s5, &r5);
  *res = cmk(s4, s5);
  *e1 = cmk(q0, q2);
  *e2 = cmk(-q1, q3);
  *e3 = cmk(r4, r5);
}
static inline void two_sum_c(cplx a, cplx b, cplx *res, cplx *err) {
  double s, e, t, f;
  two_sum(a.re, b.re, &s, &e);
  two_sum(a.im, b.im, &t, &f);
  *res = cmk(s, t);
  *err = cmk(e, f);
}
/* Priest (1992) doubly compensated summation of four terms, largest first. */
static double priest4(double p[4]) {
  for (int i = 0; i < 3; ++i) {
    int ind = i;
    double mx = fabs(p[i]);
    for (int j = i + 1; j < 4; ++j)
      if (fabs(p[j]) > mx) { mx = fabs(p[j]); ind = j; }
    if (ind != i) { double t = p[i]; p[i] = p[ind]; p[ind] = t; }
  }
  double s = p[0], c = 0;
  for (int i = 1; i < 4; ++i) {
    double y = c + p[i], u = p[i] - (y - c), t = y + s, v = y - (t - s), z = u + v;
    s = t + z;
    c = z - (s - t);
  }
  return s;
}
static cplx priest4_c(cplx a, cplx b, cplx c, cplx d) {
  double r[4] = {a.re, b.re, c.re, d.re}, i[4] = {a.im, b.im, c.im, d.im};
  return cmk(priest4(r), priest4(i));
}
static double gamma_const(unsigned n) {
  double g = (2 * n * EPS) * 1.41421356237309504880;
  return g / ((1 - DBL_EPSILON) - g);
}

/* ---- Horner evaluations (horner.h:219-267) ---- */
static double horner_real(const double *a, double x, int deg) {
  double h = a[deg];
  for (int i = deg - 1; i >= 0; --i) h = fma(h, x, a[i]);
  return h;
}
static double rhorner_real(const double *a, double x, int deg) {
  double h = a[0];
  for (int i = 1; i <= deg; ++i) h = fma(h, x, a[i]);
  return h;
}
static void horner_c(const cplx *p, cplx x, int deg, cplx *h, cplx *hd) {
  cplx H = p[deg], D = cmk(0, 0);
  for (int i = deg - 1; i >= 0; --i) {
    D = cadd(cmul(D, x), H);
    H = cadd(cmul(H, x), p[i]);
  }
  *h = H; *hd = D;
}
static void rhorner_c(const cplx *p, cplx x, int deg, cplx *h, cplx *hd) {
  cplx H = p[0], D = cmk(0, 0);
  for (int i = 1; i <= deg; ++i) {
    D = cadd(cmul(D, x), H);
    H = cadd(cmul(H, x), p[i]);
  }
  *h = H; *hd = D;
}
/* compensated Horner (horner.h:281-385); reversed=1 walks the coefficients from p[0]. */
static void horner_comp_c(const cplx *p, cplx x, int deg, int reversed, cplx *h, cplx *hd, double *eb) {
  cplx H = reversed ? p[0] : p[deg], D = cmk(0, 0), e = cmk(0, 0), ed = cmk(0, 0);
  double E = 0, ax = cabs_(x);
  for (int k = 1; k <= deg; ++k) {
    int i = reversed ? k : deg - k;
    cplx r, e1, e2, e3, se;
    two_prod_c(D, x, &r, &e1, &e2, &e3);
    two_sum_c(r, H, &D, &se);
    ed = cadd(cadd(cmul(ed, x), e), priest4_c(e1, e2, e3, se));
    two_prod_c(H, x, &r, &e1, &e2, &e3);
    two_sum_c(r, p[i], &H, &se);
    e = cadd(cmul(e, x), priest4_c(e1, e2, e3, se));
    double ap[4] = {cabs_(e1), cabs_(e2), cabs_(e3), cabs_(se)};
    E = E * ax + priest4(ap);
  }
  *h = cadd(H, e);
  *hd = cadd(D, ed);
  *eb = E;
}

/* ---- initial estimates (init_est.h:37-102) ---- */
static void init_estimates(const double *alpha, int deg, int init_mode, cplx *roots) {
  int hx[64];
  double hy[64];
  int k = 0;
  /* upper hull of (i, log alpha_i) scanning from the highest order down */
  for (int i = deg; i >= 0; --i) {
    double y = alpha[i] > 0 ? log(alpha[i]) : -1e30;
    while (k >= 2) {
      double ccw = (double)(hx[k - 1] - hx[k - 2]) * (y - hy[k - 2]) - (hy[k - 1] - hy[k - 2]) * (double)(i - hx[k - 2]);
      if (ccw <= 0) --k; else break;
    }
    hx[k] = i; hy[k] = y; ++k;
  }
  const double pi2 = 6.28318530717958647693, sigma = 0.7, th = pi2 / deg;
  int n = 0;
  for (int i = k - 2; i >= 0; --i) {
    int nz = hx[i] - hx[i + 1];
    double r = pow(alpha[hx[i + 1]], 1.0 / nz) / pow(alpha[hx[i]], 1.0 / nz);
    double ang = pi2 / nz;
    for (int j = 0; j < nz; ++j) {
      double phi = ang * j + th * i + sigma;
      roots[n + j] = init_mode == 1 ? cmk(r * sin(phi), 0.0) : cmk(r * cos(phi), r * sin(phi));
    }
    n += nz;
  }
}

static cplx aberth_sum(const cplx *z, int deg, int j) {
  cplx s = cmk(0, 0);
  for (int i = 0; i < deg; ++i)
    if (i != j) s = cadd(s, crecip(csub(z[j], z[i])));
  return s;
}
/* forward correction h / (h' - h*sum) (ehrlich_aberth.h:27-41) */
static cplx corr_fwd(const cplx *z, cplx h, cplx hd, int deg, int j) {
  return cdiv(h, csub(hd, cmul(h, aberth_sum(z, deg, j))));
}
/* z^2 as the reference forms it: thrust::pow(z, 2) = exp(2 log z)
   (ehrlich_aberth.h:56-57).  For a negative real z this leaves an O(1e-16)
   imaginary part, which is what lets real-valued iterates leave the real axis. */
static cplx csq_pow(cplx z) {
  double m = exp(2.0 * log(cabs_(z))), t = 2.0 * atan2(z.im, z.re);
  return cmk(m * cos(t), m * sin(t));
}
/* reversed-polynomial correction (ehrlich_aberth.h:43-58) */
static cplx corr_rev(const cplx *z, cplx h, cplx hd, int deg, int j) {
  cplx z2h = cmul(csq_pow(z[j]), h);
  cplx den = csub(csub(cscale(cmul(z[j], h), (double)deg), hd), cmul(z2h, aberth_sum(z, deg, j)));
  return cdiv(z2h, den);
}

static int solve_one(const cplx *p, int deg, int itmax, int compensated, const cplx *init, int init_mode,
                     cplx *z) {
  double alpha[64];
  unsigned char cx[64], cy[64];
  for (int i = 0; i <= deg; ++i) alpha[i] = cabs_(p[i]);
  if (init) for (int i = 0; i < deg; ++i) z[i] = init[i];
  else init_estimates(alpha, deg, init_mode, z);
  for (int i = 0; i <= deg; ++i) alpha[i] = alpha[i] * fma(3.8284271247461900976, i, 1);
  for (int i = 0; i < deg; ++i) cx[i] = cy[i] = 0;
  for (int it = 0; it < itmax; ++it) {
    for (int j = 0; j < deg; ++j) {
      int rev = cabs_(z[j]) > 1;
      if (!cx[j]) {
        cplx h, hd;
        double b;
        if (rev) {
          b = rhorner_real(alpha, 1.0 / cabs_(z[j]), deg);
          rhorner_c(p, crecip(z[j]), deg, &h, &hd);
        } else {
          b = horner_real(alpha, cabs_(z[j]), deg);
          horner_c(p, z[j], deg, &h, &hd);
        }
        if (cabs_(h) > EPS * b)
          z[j] = csub(z[j], rev ? corr_rev(z, h, hd, deg, j) : corr_fwd(z, h, hd, deg, j));
        else
          cx[j] = 1;
      } else if (compensated && !cy[j]) {
        cplx h, hd;
        double eb;
        horner_comp_c(p, rev ? crecip(z[j]) : z[j], deg, rev, &h, &hd, &eb);
        double ah = cabs_(h);
        double bound = EPS * ah + (gamma_const(4 * deg + 2) * eb + 2 * EPS * EPS * ah);
        if (ah > 4 * bound) {
          cplx c = rev ? corr_rev(z, h, hd, deg, j) : corr_fwd(z, h, hd, deg, j);
          double lim = rev ? 4 * EPS * cabs_(z[j]) : 4 * EPS;
          if (cabs_(c) > lim) z[j] = csub(z[j], c);
          else cy[j] = 1;
        } else {
          cy[j] = 1;
        }
      }
    }
    int all = 1;
    for (int j = 0; j < deg; ++j) all &= compensated ? cy[j] : cx[j];
    if (all) return it + 1;
  }
  return -1;
}

/* Solve `size` polynomials of degree `deg` (deg <= 63).  iters may be NULL. */
int oracle_ea_solve(int64_t size, int deg, int itmax, int compensated, int custom_init, int init_mode,
                    const double *coeffs, const double *roots_init, double *roots, int *iters) {
  if (deg < 1 || deg > 63 || size < 0) return 1;
  for (int64_t i = 0; i < size; ++i) {
    const cplx *p = (const cplx *)coeffs + i * (deg + 1);
    const cplx *init = custom_init ? (const cplx *)roots_init + i * deg : NULL;
    int it = solve_one(p, deg, itmax, compensated, init, init_mode, (cplx *)roots + i * deg);
    if (iters) iters[i] = it;
  }
  return 0;
}
