// Lens configuration and the lens-equation polynomial.
//
// Conventions follow the reference (src/caustics/point_source.py:1798-1817):
//   binary: lenses at +a (mass e1) and -a (mass 1-e1), a = s/2, e1 = 1/(1+q);
//   triple: third lens at r3*exp(i psi), e1 = q/(1+q+q3), e2 = q*e1, e3 = 1-e1-e2;
//   source positions are shifted by x_cm = a(1-q)/(1+q).
//
// The degree n^2+1 polynomial is built by eliminating conj(z) from the lens
// equation w = z - sum_j eps_j / (conj(z) - conj(r_j)):
//   D(z) = prod_j (z - r_j),  N(z) = sum_j eps_j prod_{k!=j} (z - r_k),
//   G_j(z) = (conj(w) - conj(r_j)) D(z) + N(z),
//   P(z) = (z - w) prod_j G_j - D sum_j eps_j prod_{k!=j} G_k.
// It equals, coefficient for coefficient, the reference's expanded monomial
// forms (point_source.py:17-86 and 89-1479), at a fraction of their cost.
#pragma once
#include "cplx.cuh"

struct Lens {
  int n;          // number of lenses (2 or 3)
  cd r[3];        // lens positions (complex)
  double eps[3];  // mass fractions
  double x_cm;    // centre-of-mass shift applied to source positions
  cd D[4];        // prod_j (z - r_j), low -> high
  cd N[3];        // sum_j eps_j prod_{k!=j} (z - r_k), low -> high
};

// Construction from the reference's user parameters (host or device).
__host__ __device__ inline Lens make_lens(int nlenses, double s, double q, double q3, double r3, double psi) {
  Lens L{};
  L.n = nlenses;
  double a = 0.5 * s;
  L.x_cm = a * (1.0 - q) / (1.0 + q);
  if (nlenses == 2) {
    double e1 = 1.0 / (1.0 + q);
    L.r[0] = mk(a, 0.0);
    L.r[1] = mk(-a, 0.0);
    L.eps[0] = e1;
    L.eps[1] = 1.0 - e1;
  } else {
    double e1 = q / (1.0 + q + q3);
    double e2 = q * e1;
    L.r[0] = mk(a, 0.0);
    L.r[1] = mk(-a, 0.0);
    L.r[2] = mk(r3 * cos(psi), r3 * sin(psi));
    L.eps[0] = e1;
    L.eps[1] = e2;
    L.eps[2] = 1.0 - e1 - e2;
  }
  // D = prod (z - r_j)
  cd D[4] = {mk(1, 0), mk(0, 0), mk(0, 0), mk(0, 0)};
  for (int j = 0; j < L.n; ++j) {
    cd nd[4] = {mk(0, 0), mk(0, 0), mk(0, 0), mk(0, 0)};
    for (int k = 0; k <= j; ++k) {
      nd[k + 1] = nd[k + 1] + D[k];
      nd[k] = nd[k] - D[k] * L.r[j];
    }
    for (int k = 0; k < 4; ++k) D[k] = nd[k];
  }
  cd N[3] = {mk(0, 0), mk(0, 0), mk(0, 0)};
  for (int j = 0; j < L.n; ++j) {
    cd t[3] = {mk(L.eps[j], 0), mk(0, 0), mk(0, 0)};
    int deg = 0;
    for (int k = 0; k < L.n; ++k) {
      if (k == j) continue;
      cd nt[3] = {mk(0, 0), mk(0, 0), mk(0, 0)};
      for (int i = 0; i <= deg; ++i) {
        nt[i + 1] = nt[i + 1] + t[i];
        nt[i] = nt[i] - t[i] * L.r[k];
      }
      for (int i = 0; i < 3; ++i) t[i] = nt[i];
      ++deg;
    }
    for (int i = 0; i < 3; ++i) N[i] = N[i] + t[i];
  }
  for (int k = 0; k < 4; ++k) L.D[k] = D[k];
  for (int k = 0; k < 3; ++k) L.N[k] = N[k];
  return L;
}

// Polynomial coefficients, low -> high, for source position w (already shifted).
template <int NL>
CGB_HD void lens_poly(const Lens &L, cd w, cd (&p)[NL * NL + 2]) {
  constexpr int DEG = NL * NL + 1;
  cd wb = conj(w);
  cd G[NL][NL + 1];
#pragma unroll
  for (int j = 0; j < NL; ++j) {
    cd c = wb - conj(L.r[j]);
#pragma unroll
    for (int k = 0; k <= NL; ++k) G[j][k] = (k < NL) ? cfma(c, L.D[k], L.N[k]) : c * L.D[k];
  }
  // prod_j G_j  and  S = sum_j eps_j prod_{k!=j} G_k
  constexpr int PD = NL * NL;  // degree of prod_j G_j
  cd prod[PD + 1];
  cd S[PD - NL + 1];
  if (NL == 2) {
#pragma unroll
    for (int i = 0; i <= PD; ++i) prod[i] = mk(0, 0);
#pragma unroll
    for (int i = 0; i <= NL; ++i)
#pragma unroll
      for (int k = 0; k <= NL; ++k) prod[i + k] = cfma(G[0][i], G[1][k], prod[i + k]);
#pragma unroll
    for (int i = 0; i <= NL; ++i) S[i] = G[1][i] * L.eps[0] + G[0][i] * L.eps[1];
  } else {
    cd g01[2 * NL + 1], g02[2 * NL + 1], g12[2 * NL + 1];
#pragma unroll
    for (int i = 0; i <= 2 * NL; ++i) g01[i] = g02[i] = g12[i] = mk(0, 0);
#pragma unroll
    for (int i = 0; i <= NL; ++i)
#pragma unroll
      for (int k = 0; k <= NL; ++k) {
        g01[i + k] = cfma(G[0][i], G[1][k], g01[i + k]);
        g02[i + k] = cfma(G[0][i], G[2 % NL][k], g02[i + k]);
        g12[i + k] = cfma(G[1][i], G[2 % NL][k], g12[i + k]);
      }
#pragma unroll
    for (int i = 0; i <= PD; ++i) prod[i] = mk(0, 0);
#pragma unroll
    for (int i = 0; i <= 2 * NL; ++i)
#pragma unroll
      for (int k = 0; k <= NL; ++k) prod[i + k] = cfma(g01[i], G[2 % NL][k], prod[i + k]);
#pragma unroll
    for (int i = 0; i <= 2 * NL; ++i)
      S[i] = g12[i] * L.eps[0] + g02[i] * L.eps[1] + g01[i] * L.eps[2 % NL];
  }
  // P = (z - w) prod - D S
#pragma unroll
  for (int i = 0; i <= DEG; ++i) p[i] = mk(0, 0);
#pragma unroll
  for (int i = 0; i <= PD; ++i) {
    p[i + 1] = p[i + 1] + prod[i];
    p[i] = p[i] - w * prod[i];
  }
#pragma unroll
  for (int i = 0; i <= PD - NL; ++i)
#pragma unroll
    for (int k = 0; k <= NL; ++k) p[i + k] = p[i + k] - L.D[k] * S[i];
}

// Coefficient m (0..5) of lens_poly<2>(L, w): the terms of p[m] only, added in
// the order lens_poly adds them, so that six lanes, one per coefficient, give
// lens_poly's values with a dependent chain about half as long.
CGB_HD cd lens_poly2_coef(const Lens &L, cd w, int m) {
  const cd wb = conj(w);
  cd G[2][3];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const cd c = wb - conj(L.r[j]);
#pragma unroll
    for (int k = 0; k <= 2; ++k) G[j][k] = (k < 2) ? cfma(c, L.D[k], L.N[k]) : c * L.D[k];
  }
  auto prod = [&](int n) {  // prod_j G_j, coefficient n
    cd a = mk(0, 0);
#pragma unroll
    for (int i = 0; i <= 2; ++i)
      if (n - i >= 0 && n - i <= 2) a = cfma(G[0][i], G[1][n - i], a);
    return a;
  };
  cd v = mk(0, 0);
  if (m >= 1) v = v + prod(m - 1);
  if (m <= 4) v = v - w * prod(m);
#pragma unroll
  for (int i = 0; i <= 2; ++i)
    if (m - i >= 0 && m - i <= 2) v = v - L.D[m - i] * (G[1][i] * L.eps[0] + G[0][i] * L.eps[1]);
  return v;
}

// w = z - sum_j eps_j / (conj(z) - conj(r_j))   (point_source.py:1536-1556)
template <int NL>
__device__ __forceinline__ cd lens_eq(const Lens &L, cd z) {
  cd zb = conj(z);
  cd w = z;
#pragma unroll
  for (int j = 0; j < NL; ++j) w = w - crecip(zb - conj(L.r[j])) * L.eps[j];
  return w;
}

// Image filter of one root: resid = |lens_eq(z) - w| and det = det J, with the
// reciprocals 1 / (conj(z) - conj(r_j)) shared; each quantity is accumulated in
// the same order as lens_eq and lens_det, so both agree with them bit for bit.
template <int NL>
__device__ __forceinline__ void lens_filter(const Lens &L, cd z, cd w, double &resid, double &det) {
  const cd zb = conj(z);
  cd weq = z, lam = mk(0, 0);
#pragma unroll
  for (int j = 0; j < NL; ++j) {
    const cd t = crecip(zb - conj(L.r[j]));
    weq = weq - t * L.eps[j];
    lam = lam + t * t * L.eps[j];
  }
  resid = cabs(weq - w);
  det = 1.0 - norm2(lam);
}

// det J = 1 - |sum_j eps_j / (conj(z) - conj(r_j))^2|^2   (point_source.py:1558-1580)
template <int NL>
__device__ __forceinline__ double lens_det(const Lens &L, cd z) {
  cd zb = conj(z);
  cd s = mk(0, 0);
#pragma unroll
  for (int j = 0; j < NL; ++j) {
    cd t = crecip(zb - conj(L.r[j]));
    s = s + t * t * L.eps[j];
  }
  double n = norm2(s);
  return 1.0 - n;
}
