// Complex and double-float arithmetic for the magnification kernels.
//
// cd: complex FP64, cf: complex FP32.  df: an unevaluated sum hi + lo of two
// floats ("double-float"), used by the compensated Horner evaluation of the
// mixed-precision root solver (error-free TwoSum / TwoProd via FMA).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#define CGB_HD __host__ __device__ __forceinline__

struct cd {
  double x, y;
};
struct cf {
  float x, y;
};

CGB_HD cd mk(double x, double y) { return cd{x, y}; }
CGB_HD cd operator+(cd a, cd b) { return cd{a.x + b.x, a.y + b.y}; }
CGB_HD cd operator-(cd a, cd b) { return cd{a.x - b.x, a.y - b.y}; }
CGB_HD cd operator-(cd a) { return cd{-a.x, -a.y}; }
CGB_HD cd operator*(cd a, cd b) { return cd{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
CGB_HD cd operator*(cd a, double s) { return cd{a.x * s, a.y * s}; }
CGB_HD cd operator*(double s, cd a) { return cd{a.x * s, a.y * s}; }
CGB_HD cd conj(cd a) { return cd{a.x, -a.y}; }
CGB_HD double norm2(cd a) { return a.x * a.x + a.y * a.y; }
CGB_HD double cabs(cd a) { return sqrt(a.x * a.x + a.y * a.y); }
CGB_HD cd cdiv(cd a, cd b) {
  double inv = 1.0 / (b.x * b.x + b.y * b.y);
  return cd{(a.x * b.x + a.y * b.y) * inv, (a.y * b.x - a.x * b.y) * inv};
}
CGB_HD cd crecip(cd b) {
  double inv = 1.0 / (b.x * b.x + b.y * b.y);
  return cd{b.x * inv, -b.y * inv};
}
// a*b + c with FMAs
CGB_HD cd cfma(cd a, cd b, cd c) {
  return cd{fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y))};
}

CGB_HD cf mkf(float x, float y) { return cf{x, y}; }
CGB_HD cf tof(cd a) { return cf{(float)a.x, (float)a.y}; }
CGB_HD cd tod(cf a) { return cd{(double)a.x, (double)a.y}; }
CGB_HD cf operator+(cf a, cf b) { return cf{a.x + b.x, a.y + b.y}; }
CGB_HD cf operator-(cf a, cf b) { return cf{a.x - b.x, a.y - b.y}; }
CGB_HD cf operator-(cf a) { return cf{-a.x, -a.y}; }
CGB_HD cf operator*(cf a, cf b) { return cf{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
CGB_HD cf operator*(cf a, float s) { return cf{a.x * s, a.y * s}; }
CGB_HD cf conj(cf a) { return cf{a.x, -a.y}; }
CGB_HD float norm2(cf a) { return a.x * a.x + a.y * a.y; }
CGB_HD float cabs(cf a) { return sqrtf(a.x * a.x + a.y * a.y); }
CGB_HD cf cdiv(cf a, cf b) {
  float inv = 1.0f / (b.x * b.x + b.y * b.y);
  return cf{(a.x * b.x + a.y * b.y) * inv, (a.y * b.x - a.x * b.y) * inv};
}
CGB_HD cf crecip(cf b) {
  float inv = 1.0f / (b.x * b.x + b.y * b.y);
  return cf{b.x * inv, -b.y * inv};
}
CGB_HD cf cfma(cf a, cf b, cf c) {
  return cf{fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y))};
}

// square root and absolute value in the argument's own precision (templated
// code must never widen an FP32 quantity to FP64: on GB300 the FP64 pipe is
// ~60x narrower)
CGB_HD float msqrt(float x) { return sqrtf(x); }
CGB_HD double msqrt(double x) { return sqrt(x); }
CGB_HD float mabs(float x) { return fabsf(x); }
CGB_HD double mabs(double x) { return fabs(x); }

// ---- error-free transformations (Knuth TwoSum, FMA-based TwoProd) ----
template <typename T>
CGB_HD void two_sum(T a, T b, T &s, T &e) {
  s = a + b;
  T t = s - a;
  e = (a - (s - t)) + (b - t);
}
CGB_HD void two_prod(double a, double b, double &p, double &e) {
  p = a * b;
  e = fma(a, b, -p);
}
CGB_HD void two_prod(float a, float b, float &p, float &e) {
  p = a * b;
  e = fmaf(a, b, -p);
}
