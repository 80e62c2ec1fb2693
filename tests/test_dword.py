"""Double-word arithmetic (caustics_gb300/csrc/dword.cuh) against FP64 on the
CPU: the header is compiled for the host with nvcc and each operation is
checked on random operands spanning sixteen decades.  The adjoint's
high-tangent quadrature runs on these operations under mixed precision."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include "caustics_gb300/csrc/dword.cuh"
#include <cstdio>
#include <random>
int main() {
  std::mt19937_64 g(1);
  std::uniform_real_distribution<double> U(-1.0, 1.0), E(-8, 8);
  double worst[8] = {0};
  for (int i = 0; i < 200000; ++i) {
    const double a0 = U(g) * pow(10.0, E(g)), b0 = U(g) * pow(10.0, E(g));
    const dw A(a0), B(b0);
    const double a = (double)A, b = (double)B;  // the represented values
    const double r[6] = {(double)(A + B), (double)(A - B), (double)(A * B), (double)(A / B),
                         (double)msqrt(dw(fabs(a))), (double)(A * (float)b)};
    const double e[6] = {a + b, a - b, a * b, a / b, sqrt(fabs(a)), a * (double)(float)b};
    for (int k = 0; k < 6; ++k) {
      const double den = k < 2 ? fmax(fabs(a), fabs(b)) : fabs(e[k]);
      if (den > 0) worst[k] = fmax(worst[k], fabs(r[k] - e[k]) / den);
    }
    const cdw z{A, B};
    const double n = a * a + b * b;
    const cdw rz = crecip(z);
    worst[6] = fmax(worst[6], (fabs((double)rz.x - a / n) + fabs((double)rz.y + b / n)) * sqrt(n));
    worst[7] = fmax(worst[7], fabs((double)cabs(z) - sqrt(n)) / sqrt(n));
  }
  for (int k = 0; k < 8; ++k) printf("%.3e\n", worst[k]);
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not on PATH")
def test_double_word_operations_against_fp64(tmp_path):
    src = tmp_path / "dw_check.cu"
    src.write_text(SRC)
    exe = tmp_path / "dw_check"
    subprocess.run(["nvcc", "-std=c++17", "-O2", "-I", ROOT, str(src), "-o", str(exe)], check=True,
                   capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    worst = [float(x) for x in out]
    names = ["add", "sub", "mul", "div", "sqrt", "mul_float", "crecip", "cabs"]
    # u = 2^-24: the sloppy sum is bounded by ~2u^2 (|a| + |b|) <= 4u^2 max(|a|,
    # |b|) = 1.4e-14 of the larger operand, the products by 5u^2 and 2u^2 of the
    # result (Joldes, Muller, Popescu 2017); quotient and square root by one
    # Newton step
    bounds = [1.5e-14, 1.5e-14, 2e-14, 6e-14, 3e-14, 1e-14, 6e-14, 3e-14]
    for n, w, b in zip(names, worst, bounds):
        assert w < b, (n, w)
