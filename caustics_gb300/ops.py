"""The C ABI registered as torch operators (namespace ``caustics``).

The reference registers its native root solver as XLA custom-call targets
(src/caustics/ehrlich_aberth_primitive.py:15-28, wired at :359-373) and gets
gradients from JAX autodiff.  Here the same entry points are torch custom ops,
so they are visible to ``torch.compile`` / ``torch.export`` (fake-tensor
shape functions) and differentiable through the hand-written adjoints
(``register_autograd``):

  caustics::ea_solve ................. cgb_ea_solve (backward: cgb_ea_roots_vjp)
  caustics::mag_point_source ......... cgb_mag_point_source
  caustics::mag_extended_source ...... cgb_mag_extended_source_ws
                                       (backward: cgb_mag_extended_source_grad_ws)
  caustics::mag ...................... cgb_mag_ws
  caustics::mag_lc_batched ........... cgb_mag_lc_batched (backward: cgb_mag_lc_batched_vjp)
  caustics::mag_lc_batched_vjp ....... cgb_mag_lc_batched_vjp

Each op launches on the current CUDA stream and needs CUDA tensors; like the
rest of the package there is no CPU implementation.  Precision arguments are
the C ABI's codes (0 = FP64, 1 = mixed, 2 = compensated FP64 for ea_solve).
"""
from typing import List, Optional

import torch
from torch import Tensor

from . import api as A

_PREC_NAME = {0: "fp64", 1: "mixed", 2: "fp64_comp"}


def _prec(p: int) -> str:
    if p not in _PREC_NAME:
        raise ValueError(f"precision code must be 0, 1 or 2, got {p}")
    return _PREC_NAME[p]


# ---- root solver (the ehrlich_aberth primitive) ----

@torch.library.custom_op("caustics::ea_solve", mutates_args=())
def ea_solve(coeffs: Tensor, roots_init: Optional[Tensor], itmax: int, precision: int) -> Tensor:
    """Roots [M, deg] of the polynomials coeffs [M, deg+1] (complex128, low ->
    high), warm-started from roots_init [M, deg] when given."""
    c = coeffs.contiguous()
    ri = None if roots_init is None else roots_init.reshape(c.shape[0], c.shape[1] - 1).contiguous()
    return A._solve(c, ri, itmax, A._precision(_prec(precision)), None)


@ea_solve.register_fake
def _(coeffs, roots_init, itmax, precision):
    return coeffs.new_empty((coeffs.shape[0], coeffs.shape[1] - 1))


@torch.library.custom_op("caustics::ea_roots_vjp", mutates_args=())
def ea_roots_vjp(coeffs: Tensor, roots: Tensor, ct_roots: Tensor) -> Tensor:
    """Cotangent of the coefficients from that of the roots (implicit-function
    rule, torch's conjugate convention)."""
    c, z, g = coeffs.contiguous(), roots.contiguous(), ct_roots.contiguous()
    ct = torch.empty_like(c)
    with torch.cuda.device(c.device):
        A.L.check(A.L.lib().cgb_ea_roots_vjp(A._ptr(c), A._ptr(z), A._ptr(g), A._ptr(ct), c.shape[0], c.shape[1] - 1,
                                             1, A._stream()), "cgb_ea_roots_vjp")
    return ct


@ea_roots_vjp.register_fake
def _(coeffs, roots, ct_roots):
    return torch.empty_like(coeffs)


def _ea_setup(ctx, inputs, output):
    ctx.save_for_backward(inputs[0], output)


def _ea_backward(ctx, g):
    c, z = ctx.saved_tensors
    return ea_roots_vjp(c, z, g), None, None, None


ea_solve.register_autograd(_ea_backward, setup_context=_ea_setup)


# ---- point source ----

@torch.library.custom_op("caustics::mag_point_source", mutates_args=())
def mag_point_source(w: Tensor, nlenses: int, s: float, q: float, q3: float, r3: float, psi: float, itmax: int,
                     precision: int) -> Tensor:
    """Point-source magnification of the source positions w (complex128)."""
    p = dict(s=s, q=q) if nlenses == 2 else dict(s=s, q=q, q3=q3, r3=r3, psi=psi)
    return A.mag_point_source(w.contiguous(), nlenses=nlenses, roots_itmax=itmax, precision=_prec(precision), **p)


@mag_point_source.register_fake
def _(w, nlenses, s, q, q3, r3, psi, itmax, precision):
    return w.new_empty(w.shape, dtype=torch.float64)


# ---- extended source, differentiable in w0 and the lens, source and limb parameters ----

def _es_kw(npts_limb, limb_darkening, npts_ld, itmax, precision):
    return dict(npts_limb=npts_limb, limb_darkening=limb_darkening, npts_ld=npts_ld, roots_itmax=itmax,
                precision=_prec(precision))


@torch.library.custom_op("caustics::mag_extended_source", mutates_args=())
def mag_extended_source(w0: Tensor, params: Tensor, nlenses: int, npts_limb: int, limb_darkening: bool,
                        npts_ld: int, itmax: int, precision: int) -> Tensor:
    """Extended-source magnification of the source centres w0 (complex128 [n]);
    params (float64): (s, q, rho, u1) for binary lenses, (s, q, rho, u1, q3, r3,
    psi) for triple lenses; differentiable in w0 and params."""
    pv = [float(x) for x in params.detach().cpu()]
    lens = dict(s=pv[0], q=pv[1]) if nlenses == 2 else dict(s=pv[0], q=pv[1], q3=pv[4], r3=pv[5], psi=pv[6])
    return A.mag_extended_source(w0.contiguous(), pv[2], nlenses=nlenses, u1=pv[3],
                                 **_es_kw(npts_limb, limb_darkening, npts_ld, itmax, precision), **lens)


@mag_extended_source.register_fake
def _(w0, params, nlenses, npts_limb, limb_darkening, npts_ld, itmax, precision):
    return w0.new_empty(w0.shape, dtype=torch.float64)


@torch.library.custom_op("caustics::mag_extended_source_grad", mutates_args=())
def mag_extended_source_grad(w0: Tensor, params: Tensor, npts_limb: int, limb_darkening: bool, npts_ld: int,
                             itmax: int, precision: int) -> List[Tensor]:
    """(mag [n], grad [n, k]): binary lens (params (s, q, rho, u1)), k = 6,
    grad = d mag / d(s, q, rho, u1, Re w0, Im w0); triple lens (params (s, q,
    rho, u1, q3, r3, psi)), k = 9, with d mag / d(q3, r3, psi) appended.  The
    contours are recomputed, not stored."""
    pv = [float(x) for x in params.detach().cpu()]
    lens = dict(s=pv[0], q=pv[1]) if len(pv) == 4 else dict(s=pv[0], q=pv[1], q3=pv[4], r3=pv[5], psi=pv[6])
    m, g = A.mag_extended_source_grad(w0.contiguous(), pv[2], nlenses=2 if len(pv) == 4 else 3, u1=pv[3],
                                      **_es_kw(npts_limb, limb_darkening, npts_ld, itmax, precision), **lens)
    return [m, g]


@mag_extended_source_grad.register_fake
def _(w0, params, npts_limb, limb_darkening, npts_ld, itmax, precision):
    n = w0.numel()
    k = 6 if params.shape[0] == 4 else 9
    return [w0.new_empty((n,), dtype=torch.float64), w0.new_empty((n, k), dtype=torch.float64)]


def _es_setup(ctx, inputs, output):
    w0, params, nlenses, npts_limb, limb_darkening, npts_ld, itmax, precision = inputs
    ctx.save_for_backward(w0, params)
    ctx.opts = (npts_limb, limb_darkening, npts_ld, itmax, precision)


def _es_backward(ctx, gmag):
    w0, params = ctx.saved_tensors
    _, g = mag_extended_source_grad(w0, params, *ctx.opts)
    gm = gmag.reshape(-1)
    gw = (gm * torch.complex(g[:, 4], g[:, 5])).reshape(w0.shape)
    gp = torch.zeros_like(params)
    gp[:4] = (gm[:, None] * g[:, :4]).sum(0)
    if params.shape[0] == 7:  # (q3, r3, psi)
        gp[4:] = (gm[:, None] * g[:, 6:]).sum(0)
    return gw, gp, None, None, None, None, None, None


mag_extended_source.register_autograd(_es_backward, setup_context=_es_setup)


# ---- light curve with hexadecapole routing ----

@torch.library.custom_op("caustics::mag", mutates_args=())
def mag(w: Tensor, rho: float, nlenses: int, s: float, q: float, q3: float, r3: float, psi: float, npts_limb: int,
        limb_darkening: bool, u1: float, npts_ld: int, itmax: int, precision: int) -> Tensor:
    """mag(): hexadecapole where the reference's tests accept it, contour
    integration elsewhere (every point for triple lenses, as the reference)."""
    p = dict(s=s, q=q) if nlenses == 2 else dict(s=s, q=q, q3=q3, r3=r3, psi=psi)
    return A.mag(w.contiguous(), rho, nlenses=nlenses, u1=u1, **_es_kw(npts_limb, limb_darkening, npts_ld, itmax,
                                                                           precision), **p)


@mag.register_fake
def _(w, rho, nlenses, s, q, q3, r3, psi, npts_limb, limb_darkening, u1, npts_ld, itmax, precision):
    return w.new_empty(w.shape, dtype=torch.float64)


# ---- batched light curves, differentiable in the curve parameters ----

def _lc_kw(npts_limb, limb_darkening, npts_ld, itmax, precision):
    return dict(npts_limb=npts_limb, limb_darkening=limb_darkening, npts_ld=npts_ld, roots_itmax=itmax,
                precision=_prec(precision))


@torch.library.custom_op("caustics::mag_lc_batched", mutates_args=())
def mag_lc_batched(offsets: Tensor, t: Tensor, curves: Tensor, npts_limb: int, limb_darkening: bool, npts_ld: int,
                   itmax: int, precision: int) -> Tensor:
    """Magnifications [npoints] of binary-lens light curves of uneven lengths:
    offsets int64 [ncurves+1], t float64 [npoints], curves float64 [ncurves, 8]
    = (s, q, rho, u1, u0, alpha, t0, tE)."""
    return A.mag_lc_batched(offsets, t, curves.detach(), **_lc_kw(npts_limb, limb_darkening, npts_ld, itmax,
                                                                  precision))


@mag_lc_batched.register_fake
def _(offsets, t, curves, npts_limb, limb_darkening, npts_ld, itmax, precision):
    return t.new_empty(t.shape, dtype=torch.float64)


@torch.library.custom_op("caustics::mag_lc_batched_vjp", mutates_args=())
def mag_lc_batched_vjp(offsets: Tensor, t: Tensor, curves: Tensor, cot: Tensor, npts_limb: int,
                       limb_darkening: bool, npts_ld: int, itmax: int, precision: int) -> Tensor:
    """grad [ncurves, 8] = sum over each curve's points of cot[i] d mag_i / d curves[c]."""
    g, _ = A.mag_lc_batched_vjp(offsets, t, curves.detach(), cot, **_lc_kw(npts_limb, limb_darkening, npts_ld, itmax,
                                                                           precision))
    return g


@mag_lc_batched_vjp.register_fake
def _(offsets, t, curves, cot, npts_limb, limb_darkening, npts_ld, itmax, precision):
    return torch.empty_like(curves)


def _lc_setup(ctx, inputs, output):
    offsets, t, curves = inputs[:3]
    ctx.save_for_backward(offsets, t, curves)
    ctx.opts = tuple(inputs[3:])


def _lc_backward(ctx, gmag):
    offsets, t, curves = ctx.saved_tensors
    g = mag_lc_batched_vjp(offsets, t, curves, gmag.contiguous(), *ctx.opts)
    return None, None, g, None, None, None, None, None


mag_lc_batched.register_autograd(_lc_backward, setup_context=_lc_setup)
