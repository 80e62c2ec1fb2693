// Double-word arithmetic on the FP32 pipe: a value hi + lo of two floats with
// |lo| <= ulp(hi) / 2, about 48 significant bits.  On GB300 an FP64
// instruction holds its scheduler's narrow FP64 pipe for ~64 cycles, while
// FP32 instructions issue one per cycle, so work that is throughput-bound and
// needs more than FP32 runs faster as a few FP32 operations per FP64 one.
//
// Algorithms (u = 2^-24): Knuth's TwoSum, TwoProd by FMA, and the double-word
// operations of M. Joldes, J.-M. Muller, V. Popescu, "Tight and rigorous error
// bounds for basic building blocks of double-word arithmetic", ACM TOMS 44
// (2017): the sum of two double-words in its sloppy form (error <= ~2u^2 of
// the operands' magnitudes, the bound the quadrature's FP64 form has in units
// of its own rounding; the accurate form, 3u^2 of the result, costs twice the
// instructions), the product of two double-words with FMA (<= 5u^2) and of a
// double-word by a float (<= 2u^2).  Quotient and square root take the FP32
// result and one Newton correction computed with those operations (relative
// error ~1e-13).
// Values must stay in the FP32 exponent range; the quadrature that uses them
// does (lengths and parameters of order 1e-4 .. 1e4).
#pragma once
#include "cplx.cuh"

struct dw {
  float hi, lo;
  dw() = default;
  CGB_HD constexpr dw(float h, float l) : hi(h), lo(l) {}
  CGB_HD constexpr dw(float h) : hi(h), lo(0.0f) {}
  CGB_HD constexpr dw(int h) : hi((float)h), lo(0.0f) {}
  // from FP64 (setup code; constants fold at compile time)
  CGB_HD explicit dw(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
  CGB_HD explicit operator double() const { return (double)hi + (double)lo; }
};

// approximate FP32 quotient (a few ulp); the Newton corrections absorb it
CGB_HD float dw_qdiv(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdividef(a, b);
#else
  return a / b;
#endif
}
CGB_HD dw dw_fast_two_sum(float a, float b) {  // |a| >= |b| (or a == 0)
  const float s = a + b;
  return dw(s, b - (s - a));
}
CGB_HD dw dw_two_sum(float a, float b) {
  const float s = a + b;
  const float t = s - a;
  return dw(s, (a - (s - t)) + (b - t));
}
// Sum of two double-words: TwoSum of the high parts, the low parts added in
// FP32 (the "sloppy" sum).  Its error is at most ~2u^2 (|x| + |y|): relative
// to the operands, not the result, as FP64's own rounding of a sum is bounded
// by u64 |x + y| only for the result of one operation, and u^2 = 2^-48.
CGB_HD dw operator+(dw x, dw y) {
  const dw s = dw_two_sum(x.hi, y.hi);
  return dw_fast_two_sum(s.hi, s.lo + (x.lo + y.lo));
}
CGB_HD dw operator-(dw x) { return dw(-x.hi, -x.lo); }
CGB_HD dw operator-(dw x, dw y) { return x + (-y); }
CGB_HD dw operator*(dw x, dw y) {
  const float ch = x.hi * y.hi, cl1 = fmaf(x.hi, y.hi, -ch);
  const float tl = fmaf(x.hi, y.lo, x.lo * y.lo);
  const float cl2 = fmaf(x.lo, y.hi, tl);
  return dw_fast_two_sum(ch, cl1 + cl2);
}
CGB_HD dw operator*(dw x, float y) {
  const float ch = x.hi * y, cl1 = fmaf(x.hi, y, -ch);
  const dw t = dw_fast_two_sum(ch, x.lo * y);
  return dw_fast_two_sum(t.hi, t.lo + cl1);
}
CGB_HD dw operator*(float y, dw x) { return x * y; }
CGB_HD dw operator/(dw x, dw y) {
  const float q = dw_qdiv(x.hi, y.hi);
  const dw r = x - y * q;  // y q to 2u^2: the residual is exact to ~u^3 |x|
  return dw_fast_two_sum(q, dw_qdiv(r.hi, y.hi));
}
CGB_HD dw &operator+=(dw &x, dw y) { return x = x + y; }
CGB_HD bool operator>=(dw x, dw y) { return (x - y).hi >= 0.0f; }
CGB_HD bool operator>(dw x, dw y) { return (x - y).hi > 0.0f; }
CGB_HD dw msqrt(dw x) {
  if (!(x.hi > 0.0f)) return dw(sqrtf(x.hi));  // 0, or NaN for negative input
  const float s = sqrtf(x.hi);
  const float p = s * s, e = fmaf(s, s, -p);
  const dw r = x - dw(p, e);  // x - s^2
  return dw_fast_two_sum(s, dw_qdiv(r.hi, 2.0f * s));
}

struct cdw {
  dw x, y;
};
CGB_HD cdw operator+(cdw a, cdw b) { return cdw{a.x + b.x, a.y + b.y}; }
CGB_HD cdw operator-(cdw a, cdw b) { return cdw{a.x - b.x, a.y - b.y}; }
CGB_HD cdw operator*(cdw a, cdw b) { return cdw{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
CGB_HD cdw operator*(cdw a, dw s) { return cdw{a.x * s, a.y * s}; }
CGB_HD dw norm2(cdw a) { return a.x * a.x + a.y * a.y; }
CGB_HD dw cabs(cdw a) { return msqrt(norm2(a)); }
CGB_HD cdw crecip(cdw b) {
  const dw inv = dw(1.0f) / norm2(b);
  return cdw{b.x * inv, -(b.y * inv)};
}
