"""The binary lens polynomial built one coefficient per lane
(lens_poly2_coef in caustics_gb300/csrc/lens.cuh, used by the contour kernel's
refinement) against the whole-polynomial builder lens_poly<2> and the
oracle's polynomial, on the CPU: the header is compiled for the host with
nvcc.  The per-coefficient form adds each coefficient's terms in lens_poly's
order, so the two agree bit for bit; both agree with the oracle to 1e-13 of
the coefficients' scale."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import caustics_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include "caustics_gb300/csrc/lens.cuh"
#include <cstdio>
#include <cstdlib>
int main(int argc, char **argv) {
  const Lens L = make_lens(2, atof(argv[1]), atof(argv[2]), 0.0, 0.0, 0.0);
  double wx, wy;
  while (scanf("%lf %lf", &wx, &wy) == 2) {
    cd p[6];
    lens_poly<2>(L, mk(wx, wy), p);
    int same = 1;
    for (int m = 0; m < 6; ++m) {
      const cd c = lens_poly2_coef(L, mk(wx, wy), m);
      same &= (c.x == p[m].x) && (c.y == p[m].y);
    }
    printf("%d", same);
    for (int m = 0; m < 6; ++m) printf(" %.17g %.17g", p[m].x, p[m].y);
    printf("\n");
  }
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not on PATH")
def test_per_coefficient_binary_polynomial(tmp_path):
    src = tmp_path / "lens_coef_check.cu"
    src.write_text(SRC)
    exe = tmp_path / "lens_coef_check"
    subprocess.run(["nvcc", "-std=c++17", "-O2", "-I", ROOT, str(src), "-o", str(exe)], check=True,
                   capture_output=True)
    rng = np.random.default_rng(5)
    for s, q in ((0.9, 0.1), (1.1, 5e-3), (0.4, 1e-4), (2.5, 0.7)):
        w = rng.uniform(-1.5, 1.5, 300) + 1j * rng.uniform(-1.5, 1.5, 300)
        inp = "".join(f"{float(x.real)!r} {float(x.imag)!r}\n" for x in w)
        out = subprocess.run([str(exe), repr(s), repr(q)], input=inp, check=True, capture_output=True,
                             text=True).stdout.split("\n")
        rows = np.array([[float(v) for v in line.split()] for line in out if line.strip()])
        assert rows[:, 0].all(), (s, q)  # bit-identical to lens_poly<2>
        got = rows[:, 1::2] + 1j * rows[:, 2::2]  # low -> high
        lens = O.Lens.binary(s, q)
        ref = np.array([O.lens_polynomial(x, lens)[::-1] for x in w])
        err = (np.abs(got - ref) / np.abs(ref).max(axis=1, keepdims=True)).max()
        assert err < 1e-13, (s, q, err)
