// Hexadecapole approximation (src/caustics/multipole.py:8-244) and the
// caustic-proximity / planetary-caustic tests (src/caustics/lightcurve.py:23-85).
//
// Instead of hand-expanded recursions, the image position is written as a
// bivariate Taylor series in the source offset (x, y):
//   z = z0 + sum_{1<=k+l<=5} c_kl x^k y^l,   w = z - conj(W1(z)),  W_k = W1^{(k-1)}
// Matching orders gives c_kl(1 - ...) from
//   a_kl - conj(W2) conj(a_kl) = conj(Q_kl),  a_kl = k! l! c_kl,
// where Q_kl is the order-(k+l) coefficient of sum_{m>=2} W_{m+1}/m! delta^m
// (delta = z - z0, using lower orders only).  The signed image area
// A(rho) = 1/2 int Im(conj(z) dz/dphi) dphi over z(rho cos phi, rho sin phi)
// expands as pi*(mu0 rho^2 + dquad rho^2... ) and gives mu0, the quadrupole and
// the hexadecapole terms exactly as the reference's Cassan (2017) expressions.
#pragma once
#include "cplx.cuh"
#include "lens.cuh"

namespace hexa {

constexpr int ORD = 5;
constexpr int NC = (ORD + 1) * (ORD + 2) / 2;  // monomials with k + l <= 5
__host__ __device__ constexpr int idx(int k, int l) { return (k + l) * (k + l + 1) / 2 + l; }
// int_0^{2 pi} cos^i sin^j dphi = 2 pi (i-1)!! (j-1)!! / (i+j)!! for even i, j; else 0
__host__ __device__ inline double trig_moment(int i, int j) {
  if ((i & 1) || (j & 1)) return 0.0;
  double v = 6.283185307179586476925;
  for (int k = i - 1; k > 0; k -= 2) v *= k;
  for (int k = j - 1; k > 0; k -= 2) v *= k;
  for (int k = i + j; k > 0; k -= 2) v /= k;
  return v;
}

__device__ __forceinline__ double kfact(int n) {
  double v = 1.0;
  for (int k = 2; k <= n; ++k) v *= k;
  return v;
}

// Per-image (mu0, dquad, dhex); gamma_ld = 2 u1 / (3 - u1) (0 in the light-curve driver).
// The series state (about 140 complex numbers) lives in thread-local memory:
// it is touched once per real image, so L1-resident local arrays beat spilling
// a fully unrolled register version.
static __device__ __noinline__ void terms(const cd (&W)[5], double rho, double gamma_ld, double &mu0, double &dq,
                                   double &dh) {
  cd c[NC];            // monomial coefficients of delta = z - z0
  cd pw[ORD - 1][NC];  // pw[m-2] = delta^m, m = 2..5, filled order by order
  for (int i = 0; i < NC; ++i) {
    c[i] = mk(0, 0);
    for (int m = 0; m < ORD - 1; ++m) pw[m][i] = mk(0, 0);
  }
  const cd W2c = conj(W[0]);
  const double m0 = 1.0 / (1.0 - norm2(W[0]));
  c[idx(1, 0)] = (mk(1, 0) + W2c) * m0;
  c[idx(0, 1)] = mk(0, 1) * (mk(1, 0) - W2c) * m0;
  for (int p = 2; p <= ORD; ++p) {
    for (int m = 2; m <= p; ++m) {
      for (int l = 0; l <= p; ++l) {
        cd acc = mk(0, 0);
        for (int p1 = m - 1; p1 <= p - 1; ++p1) {
          const int p2 = p - p1;
          const int lo = max(0, l - p2), hi = min(p1, l);
          for (int l1 = lo; l1 <= hi; ++l1) {
            const int l2 = l - l1;
            cd lhs = (m == 2) ? c[idx(p1 - l1, l1)] : pw[m - 3][idx(p1 - l1, l1)];
            acc = cfma(lhs, c[idx(p2 - l2, l2)], acc);
          }
        }
        pw[m - 2][idx(p - l, l)] = acc;
      }
    }
    for (int l = 0; l <= p; ++l) {
      const int k = p - l;
      cd Q = mk(0, 0);
      for (int m = 2; m <= p; ++m) Q = Q + W[m - 1] * pw[m - 2][idx(k, l)] * (1.0 / kfact(m));
      Q = Q * (kfact(k) * kfact(l));
      cd a = (conj(Q) + W2c * Q) * m0;
      c[idx(k, l)] = a * (1.0 / (kfact(k) * kfact(l)));
    }
  }
  // area coefficients A_m = 1/(2 pi) int Im(conj(Z_p) dZ_q/dphi), p + q = m
  double A[3];
  for (int mi = 0; mi < 3; ++mi) {
    const int m = 2 + 2 * mi;
    double acc = 0.0;
    for (int p = max(1, m - ORD); p <= min(ORD, m - 1); ++p) {
      const int q = m - p;
      for (int lp = 0; lp <= p; ++lp)
        for (int lq = 0; lq <= q; ++lq) {
          const int kp = p - lp, kq = q - lq;
          double t = 0.0;
          if (kq > 0) t -= kq * trig_moment(kp + kq - 1, lp + lq + 1);
          if (lq > 0) t += lq * trig_moment(kp + kq + 1, lp + lq - 1);
          if (t != 0.0) {
            cd a = c[idx(kp, lp)], b = c[idx(kq, lq)];
            acc += (a.x * b.y - a.y * b.x) * t;  // Im(conj(a) b) t
          }
        }
    }
    A[mi] = 0.5 * acc / 3.14159265358979323846;
  }
  mu0 = A[0];
  dq = A[1] * (1.0 - gamma_ld / 5.0) * rho * rho;
  dh = A[2] * (1.0 - 11.0 * gamma_ld / 35.0) * rho * rho * rho * rho;
}

// W_k = (-1)^(k-1) (k-1)! sum_j eps_j / (z - r_j)^k, k = 2..6 (multipole.py:210-229)
template <int NL>
__device__ __forceinline__ void wk(const Lens &L, cd z, cd (&W)[5]) {
#pragma unroll
  for (int k = 0; k < 5; ++k) W[k] = mk(0, 0);
#pragma unroll
  for (int j = 0; j < NL; ++j) {
    cd u = crecip(z - L.r[j]);
    cd pw = u * u;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      W[k] = W[k] + pw * L.eps[j];
      pw = pw * u;
    }
  }
  // signs and factorials: k=2: -1, 3: +2, 4: -6, 5: +24, 6: -120
  W[0] = W[0] * -1.0;
  W[1] = W[1] * 2.0;
  W[2] = W[2] * -6.0;
  W[3] = W[3] * 24.0;
  W[4] = W[4] * -120.0;
}

// Forward-mode tangent of terms(): given dW (the tangents of W2..W6) and drho,
// returns the tangents of (mu0, dquad, dhex), differentiating the same series
// construction (product rule through the powers of delta, the a_kl solve and the
// area integrals).  One tangent direction per call.
static __device__ __noinline__ void terms_tangent(const cd (&W)[5], const cd (&dW)[5], double rho, double drho,
                                                  double gamma_ld, double &dmu0, double &ddq, double &ddh) {
  cd c[NC], dc[NC];
  cd pw[ORD - 1][NC], dpw[ORD - 1][NC];
  for (int i = 0; i < NC; ++i) {
    c[i] = dc[i] = mk(0, 0);
    for (int m = 0; m < ORD - 1; ++m) pw[m][i] = dpw[m][i] = mk(0, 0);
  }
  const cd W2c = conj(W[0]), dW2c = conj(dW[0]);
  const double m0 = 1.0 / (1.0 - norm2(W[0]));
  const double dm0 = m0 * m0 * 2.0 * (W[0].x * dW[0].x + W[0].y * dW[0].y);
  c[idx(1, 0)] = (mk(1, 0) + W2c) * m0;
  dc[idx(1, 0)] = dW2c * m0 + (mk(1, 0) + W2c) * dm0;
  c[idx(0, 1)] = mk(0, 1) * (mk(1, 0) - W2c) * m0;
  dc[idx(0, 1)] = mk(0, 1) * ((mk(0, 0) - dW2c) * m0 + (mk(1, 0) - W2c) * dm0);
  for (int p = 2; p <= ORD; ++p) {
    for (int m = 2; m <= p; ++m) {
      for (int l = 0; l <= p; ++l) {
        cd acc = mk(0, 0), dacc = mk(0, 0);
        for (int p1 = m - 1; p1 <= p - 1; ++p1) {
          const int p2 = p - p1;
          const int lo = max(0, l - p2), hi = min(p1, l);
          for (int l1 = lo; l1 <= hi; ++l1) {
            const int l2 = l - l1;
            const cd lhs = (m == 2) ? c[idx(p1 - l1, l1)] : pw[m - 3][idx(p1 - l1, l1)];
            const cd dlhs = (m == 2) ? dc[idx(p1 - l1, l1)] : dpw[m - 3][idx(p1 - l1, l1)];
            const cd r = c[idx(p2 - l2, l2)], dr = dc[idx(p2 - l2, l2)];
            acc = cfma(lhs, r, acc);
            dacc = cfma(dlhs, r, cfma(lhs, dr, dacc));
          }
        }
        pw[m - 2][idx(p - l, l)] = acc;
        dpw[m - 2][idx(p - l, l)] = dacc;
      }
    }
    for (int l = 0; l <= p; ++l) {
      const int k = p - l;
      cd Q = mk(0, 0), dQ = mk(0, 0);
      for (int m = 2; m <= p; ++m) {
        const double f = 1.0 / kfact(m);
        Q = Q + W[m - 1] * pw[m - 2][idx(k, l)] * f;
        dQ = dQ + (dW[m - 1] * pw[m - 2][idx(k, l)] + W[m - 1] * dpw[m - 2][idx(k, l)]) * f;
      }
      const double kl = kfact(k) * kfact(l);
      Q = Q * kl;
      dQ = dQ * kl;
      const cd base = conj(Q) + W2c * Q;
      const cd dbase = conj(dQ) + dW2c * Q + W2c * dQ;
      c[idx(k, l)] = base * (m0 / kl);
      dc[idx(k, l)] = (dbase * m0 + base * dm0) * (1.0 / kl);
    }
  }
  double A[3], dA[3];
  for (int mi = 0; mi < 3; ++mi) {
    const int m = 2 + 2 * mi;
    double acc = 0.0, dacc = 0.0;
    for (int p = max(1, m - ORD); p <= min(ORD, m - 1); ++p) {
      const int q = m - p;
      for (int lp = 0; lp <= p; ++lp)
        for (int lq = 0; lq <= q; ++lq) {
          const int kp = p - lp, kq = q - lq;
          double t = 0.0;
          if (kq > 0) t -= kq * trig_moment(kp + kq - 1, lp + lq + 1);
          if (lq > 0) t += lq * trig_moment(kp + kq + 1, lp + lq - 1);
          if (t != 0.0) {
            const cd a = c[idx(kp, lp)], b = c[idx(kq, lq)], da = dc[idx(kp, lp)], db = dc[idx(kq, lq)];
            acc += (a.x * b.y - a.y * b.x) * t;
            dacc += ((da.x * b.y - da.y * b.x) + (a.x * db.y - a.y * db.x)) * t;
          }
        }
    }
    A[mi] = 0.5 * acc / 3.14159265358979323846;
    dA[mi] = 0.5 * dacc / 3.14159265358979323846;
  }
  dmu0 = dA[0];
  const double fq = (1.0 - gamma_ld / 5.0), fh = (1.0 - 11.0 * gamma_ld / 35.0);
  ddq = fq * (dA[1] * rho * rho + A[1] * 2.0 * rho * drho);
  ddh = fh * (dA[2] * rho * rho * rho * rho + A[2] * 4.0 * rho * rho * rho * drho);
}

// Tangent of W_k (k = 2..6) of a binary lens along (dz, da, de1):
// W_k = c_k [e1 (z - a)^-k + (1 - e1) (z + a)^-k], c_k = (-1)^(k-1) (k-1)!.
__device__ __forceinline__ void wk_tangent_binary(const Lens &L, cd z, cd dz, double da, double de1, cd (&dW)[5]) {
  const double a = L.r[0].x, e1 = L.eps[0], e2 = L.eps[1];
  const cd u = crecip(z - mk(a, 0)), v = crecip(z + mk(a, 0));
  cd pu = u, pv = v;  // u^(k-1), v^(k-1) at k = 2
  const double ck[5] = {-1.0, 2.0, -6.0, 24.0, -120.0};
  for (int k = 0; k < 5; ++k) {
    const int m = k + 2;
    const cd um = pu * u, vm = pv * v;          // u^m, v^m
    const cd um1 = um * u, vm1 = vm * v;        // u^(m+1), v^(m+1)
    // d[(z - a)^-m] = -m (z - a)^-(m+1) (dz - da); d[(z + a)^-m] = -m (z + a)^-(m+1) (dz + da)
    const cd t = (um - vm) * de1 + um1 * (dz - mk(da, 0)) * (-(double)m * e1) + vm1 * (dz + mk(da, 0)) * (-(double)m * e2);
    dW[k] = t * ck[k];
    pu = um;
    pv = vm;
  }
}

}  // namespace hexa

// Binary-lens proximity test (lightcurve.py:23-75) with c_m=1e-2, gamma=0.02,
// c_f=4, rho_min=1e-3; z/mask over DEG=5 images of shifted source w.
__device__ __forceinline__ bool proximity_test_binary(const Lens &L, cd w, const cd (&z)[5], uint32_t mask,
                                                      double rho, double delta_mu) {
  const double a = L.r[0].x, e1 = L.eps[0], e2 = L.eps[1];
  const double c_m = 1e-2, gam = 0.02, c_f = 4.0, rho_min = 1e-3;
  auto f = [&](cd u) { return (crecip(u - mk(a, 0)) * e1 + crecip(u + mk(a, 0)) * e2) * -1.0; };
  auto fp = [&](cd u) {
    cd p = crecip(u - mk(a, 0)), m = crecip(u + mk(a, 0));
    return p * p * e1 + m * m * e2;
  };
  auto fpp = [&](cd u) {
    cd p = crecip(mk(a, 0) - u), m = crecip(mk(a, 0) + u);
    return (p * p * p * e1 - m * m * m * e2) * 2.0;
  };
  double cusp = 0.0, fac = 0.0;
  int nfalse = 0;
  const double rr = (rho + rho_min) * (rho + rho_min);
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    cd zb = conj(z[i]);
    cd zh = conj(w) - f(z[i]);
    cd fpz = fp(z[i]), fppz = fpp(z[i]), fpzb = fp(zb), fpzh = fp(zh), fppzb = fpp(zb);
    double J = 1.0 - cabs(fpz * fpzb);
    bool real = (mask >> i) & 1u;
    if (real) {
      cd t = fpzb * fpzb * fpzb * fppz * fppz * 3.0;
      double J5 = J * J * J * J * J;
      cusp += fabs(6.0 * t.y / J5 * rr);
    } else {
      ++nfalse;
      double Jh = 1.0 - cabs(fpz * fpzh);
      cd den = fppzb * fpz * Jh - fppz * fpzb * fpzh * Jh;
      fac += cabs(cdiv(mk(J * Jh * Jh, 0), den));
    }
  }
  bool t_mc = gam * cusp + delta_mu < c_m;
  bool t_f = (nfalse == 0) ? true : (0.5 * fac > c_f * (rho + rho_min));
  return t_f && t_mc;
}

// Triple-lens proximity test (the nlenses == 3 branch of lightcurve.py:23-75),
// same constants and structure as the binary one over the 10 images.
// as_written: the reference's f, f', f'' as it writes them (third-lens terms
// at -r3, f'' third term e3/(z+r3)^3); otherwise the third lens at r3 (where
// the lens equation and the hexadecapole put it) and f'' = -2 sum_j eps_j /
// (z - r_j)^3.
__device__ __forceinline__ bool proximity_test_triple(const Lens &L, cd w, const cd (&z)[10], uint32_t mask,
                                                      double rho, double delta_mu, bool as_written) {
  const double a = L.r[0].x, e1 = L.eps[0], e2 = L.eps[1], e3 = L.eps[2];
  const cd r3 = as_written ? mk(-L.r[2].x, -L.r[2].y) : L.r[2];  // the test's third-lens position
  const double c3 = as_written ? 1.0 : -2.0;                      // its f'' coefficient
  const double c_m = 1e-2, gam = 0.02, c_f = 4.0, rho_min = 1e-3;
  auto f = [&](cd u) {
    return (crecip(u - mk(a, 0)) * e1 + crecip(u + mk(a, 0)) * e2 + crecip(u - r3) * e3) * -1.0;
  };
  auto fp = [&](cd u) {
    cd p = crecip(u - mk(a, 0)), m = crecip(u + mk(a, 0)), t = crecip(u - r3);
    return p * p * e1 + m * m * e2 + t * t * e3;
  };
  auto fpp = [&](cd u) {
    cd p = crecip(mk(a, 0) - u), m = crecip(mk(a, 0) + u), t = crecip(u - r3);
    return (p * p * p * e1 - m * m * m * e2) * 2.0 + t * t * t * (c3 * e3);
  };
  double cusp = 0.0, fac = 0.0;
  int nfalse = 0;
  const double rr = (rho + rho_min) * (rho + rho_min);
#pragma unroll 1
  for (int i = 0; i < 10; ++i) {
    cd zb = conj(z[i]);
    cd zh = conj(w) - f(z[i]);
    cd fpz = fp(z[i]), fppz = fpp(z[i]), fpzb = fp(zb), fpzh = fp(zh), fppzb = fpp(zb);
    double J = 1.0 - cabs(fpz * fpzb);
    bool real = (mask >> i) & 1u;
    if (real) {
      cd t = fpzb * fpzb * fpzb * fppz * fppz * 3.0;
      double J5 = J * J * J * J * J;
      cusp += fabs(6.0 * t.y / J5 * rr);
    } else {
      ++nfalse;
      double Jh = 1.0 - cabs(fpz * fpzh);
      cd den = fppzb * fpz * Jh - fppz * fpzb * fpzh * Jh;
      fac += cabs(cdiv(mk(J * Jh * Jh, 0), den));
    }
  }
  bool t_mc = gam * cusp + delta_mu < c_m;
  bool t_f = (nfalse == 0) ? true : (0.5 * fac > c_f * (rho + rho_min));
  return t_f && t_mc;
}

// lightcurve.py:78-85, with q' = e1/(1-e1) (the inverse of q, as in the reference)
__device__ __forceinline__ bool planetary_test(const Lens &L, cd w, double rho) {
  const double a = L.r[0].x, e1 = L.eps[0];
  const double s = 2 * a, q = e1 / (1 - e1);
  const double wpc = -1.0 / s, dpc = 3.0 * sqrt(q) / s;
  double dx = wpc - w.x, dy = -w.y;
  return dx * dx + dy * dy > 2.0 * (rho * rho + dpc * dpc);
}
