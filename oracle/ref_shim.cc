// Test infrastructure only: a C-ABI wrapper around the reference's own
// header-only Ehrlich-Aberth solver (lib/ehrlich_aberth/ehrlich_aberth.h of
// fbartolic/caustics), compiled from the reference sources where they lie by
// oracle/Makefile into oracle/_ref/libref_ea.so.  The loop mirrors the XLA CPU
// custom call cpu_ehrlich_aberth (lib/ehrlich_aberth/cpu_ops.cc:15-81): one
// serial pass over the polynomials with per-call scratch.  It is used to pin
// the oracle restatement and to generate golden fixtures; nothing in the
// product links it.
#include <cstdint>
#include <vector>

#include "ehrlich_aberth.h"

extern "C" {

// coeffs: complex128[size, deg+1] low->high; roots_init/roots: complex128[size, deg].
int ref_ea_solve(int size, int deg, int itmax, int compensated, int custom_init,
                 const double *coeffs, const double *roots_init, double *roots) {
  using ehrlich_aberth_jax::point;
  using ehrlich_aberth_jax::point_conv;
  if (size < 0 || deg < 1) return 1;
  std::vector<double> alpha(deg + 1);
  std::vector<char> conv_storage(deg);
  std::vector<point_conv> conv2(deg);
  std::vector<point> pts(deg + 1), hull(deg + 1);
  const complex *c = reinterpret_cast<const complex *>(coeffs);
  const complex *ri = reinterpret_cast<const complex *>(roots_init);
  complex *r = reinterpret_cast<complex *>(roots);
  bool *conv = reinterpret_cast<bool *>(conv_storage.data());
  for (int i = 0; i < size; ++i) {
    const complex *init = custom_init ? ri + (int64_t)i * deg : nullptr;
    if (compensated)
      ehrlich_aberth_jax::ehrlich_aberth_comp(deg, itmax, custom_init != 0, c + (int64_t)i * (deg + 1),
                                              init, r + (int64_t)i * deg, alpha.data(), conv2.data(),
                                              pts.data(), hull.data());
    else
      ehrlich_aberth_jax::ehrlich_aberth(deg, itmax, custom_init != 0, c + (int64_t)i * (deg + 1), init,
                                         r + (int64_t)i * deg, alpha.data(), conv, pts.data(),
                                         hull.data());
  }
  return 0;
}

}  // extern "C"
