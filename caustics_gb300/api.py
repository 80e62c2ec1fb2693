"""Drop-in magnification API with the reference's signatures, on CUDA tensors.

Signature parity with fbartolic/caustics:
  poly_roots / ehrlich_aberth ... src/caustics/ehrlich_aberth_primitive.py:34-106
  mag_point_source .............. src/caustics/point_source.py:1763
  mag_extended_source ........... src/caustics/extended_source.py:741-752
  mag ........................... src/caustics/lightcurve.py:99-110
  lens_eq, lens_eq_det_jac ...... src/caustics/point_source.py:1536-1580
  critical_and_caustic_curves ... src/caustics/point_source.py:1582-1649
  marginalized_log_likelihood ... src/caustics/linalg.py:10-94
  AnnualParallaxTrajectory ...... src/caustics/trajectory.py:12-157

Inputs may be torch tensors (any device; CUDA tensors stay on their device)
or array-likes (copied to the current CUDA device; NumPy out).  Every
computation runs in libcaustics_gb300 on the current torch CUDA stream.
Extra keyword ``precision`` selects "fp64" (the reference's arithmetic,
default) or "mixed" (FP32 iterations with FP64 polish / accumulation).
"""
import math

import numpy as np
import torch

from . import _lib as L

_PREC = {"fp64": L.PREC_FP64, "mixed": L.PREC_MIXED, "fp64_comp": L.PREC_FP64_COMP}


def _stream():
    return ctypes_void(torch.cuda.current_stream().cuda_stream)


def ctypes_void(x):
    import ctypes
    return ctypes.c_void_p(int(x))


def _ptr(t):
    import ctypes
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else ctypes.c_void_p(0)


def _to_device(x, dtype):
    was_numpy = not isinstance(x, torch.Tensor)
    if was_numpy:
        if not torch.cuda.is_available():
            raise L.CausticsError("caustics_gb300 needs a CUDA device (no CPU fallback)")
        t = torch.as_tensor(np.asarray(x), dtype=dtype).cuda()
    else:
        if not x.is_cuda:
            if not torch.cuda.is_available():
                raise L.CausticsError("caustics_gb300 needs a CUDA device (no CPU fallback)")
            x = x.cuda()
        t = x.to(dtype)
    return t.contiguous(), was_numpy


def _out(t, was_numpy):
    return t.cpu().numpy() if was_numpy else t


def _precision(p):
    if p not in _PREC:
        raise ValueError(f"precision must be one of {sorted(_PREC)}")
    return _PREC[p]


# ---------------------------------------------------------------------------
# root solver primitive
# ---------------------------------------------------------------------------

def _solve(c, ri, itmax, prec, status):
    m, n1 = c.shape
    roots = torch.empty((m, n1 - 1), dtype=torch.complex128, device=c.device)
    with torch.cuda.device(c.device):
        L.check(L.lib().cgb_ea_solve(_ptr(c), _ptr(ri), _ptr(roots), m, n1 - 1, int(itmax or 2000), prec,
                                     _ptr(status), _stream()), "cgb_ea_solve")
    return roots


class _Roots(torch.autograd.Function):
    """Roots with the implicit-function rule as backward
    (ehrlich_aberth_primitive.py:252-312; torch's conjugate convention)."""

    @staticmethod
    def forward(ctx, c, ri, itmax, prec, status):
        roots = _solve(c, ri, itmax, prec, status)
        ctx.save_for_backward(c, roots)
        return roots

    @staticmethod
    def backward(ctx, g):
        c, roots = ctx.saved_tensors
        ct = torch.empty_like(c)
        g = g.contiguous()
        with torch.cuda.device(c.device):
            L.check(L.lib().cgb_ea_roots_vjp(_ptr(c), _ptr(roots), _ptr(g), _ptr(ct), c.shape[0], c.shape[1] - 1, 1,
                                             _stream()), "cgb_ea_roots_vjp")
        return ct, None, None, None, None


def ehrlich_aberth(coeffs, roots_init, itmax=None, compensated=None, custom_init=False, precision=None, status=None):
    """Batched primitive: coeffs complex128 [M, deg+1] low->high, roots_init
    [M, deg]; returns roots [M*deg] (ehrlich_aberth_primitive.py:98-106).
    Differentiable with respect to coeffs (torch autograd)."""
    c, was_np = _to_device(coeffs, torch.complex128)
    m, n1 = c.shape
    deg = n1 - 1
    ri = None
    if custom_init:
        ri, _ = _to_device(roots_init, torch.complex128)
        ri = ri.reshape(m, deg).contiguous()
    prec = _precision(precision) if precision else (L.PREC_FP64_COMP if compensated else L.PREC_FP64)
    if c.requires_grad:
        roots = _Roots.apply(c, ri, itmax, prec, status)
    else:
        roots = _solve(c, ri, itmax, prec, status)
    return _out(roots.reshape(-1), was_np)


def roots_jvp(coeffs, roots, dcoeffs):
    """Forward-mode derivative of the roots (the primitive's JVP rule,
    ehrlich_aberth_primitive.py:252-312): coeffs, dcoeffs [M, deg+1] low->high,
    roots [M, deg] -> droots [M, deg]."""
    c, was_np = _to_device(coeffs, torch.complex128)
    z, _ = _to_device(roots, torch.complex128)
    dc, _ = _to_device(dcoeffs, torch.complex128)
    m, n1 = c.shape
    z = z.reshape(m, n1 - 1).contiguous()
    dz = torch.empty_like(z)
    with torch.cuda.device(c.device):
        L.check(L.lib().cgb_ea_roots_jvp(_ptr(c), _ptr(z), _ptr(dc.reshape(m, n1).contiguous()), _ptr(dz), m, n1 - 1,
                                         _stream()), "cgb_ea_roots_jvp")
    return _out(dz, was_np)


def roots_vjp(coeffs, roots, ct_roots, conjugate=False):
    """Reverse-mode derivative of the roots: ct_roots [M, deg] -> ct_coeffs
    [M, deg+1], the transpose of roots_jvp's map (conjugate transpose when
    conjugate=True)."""
    c, was_np = _to_device(coeffs, torch.complex128)
    z, _ = _to_device(roots, torch.complex128)
    ct, _ = _to_device(ct_roots, torch.complex128)
    m, n1 = c.shape
    out = torch.empty_like(c)
    with torch.cuda.device(c.device):
        L.check(L.lib().cgb_ea_roots_vjp(_ptr(c), _ptr(z.reshape(m, n1 - 1).contiguous()),
                                         _ptr(ct.reshape(m, n1 - 1).contiguous()), _ptr(out), m, n1 - 1,
                                         int(bool(conjugate)), _stream()), "cgb_ea_roots_vjp")
    return _out(out, was_np)


def poly_roots(coeffs, itmax=2000, compensated=False, custom_init=False, roots_init=None, precision=None):
    """Roots of complex polynomials whose last axis holds the coefficients,
    highest order first (ehrlich_aberth_primitive.py:34-94)."""
    c, was_np = _to_device(coeffs, torch.complex128)
    ncoeffs = c.shape[-1]
    out_shape = tuple(c.shape[:-1]) + (ncoeffs - 1,)
    flat = c.reshape(-1, ncoeffs).flip(-1).contiguous()
    r = ehrlich_aberth(flat, roots_init, itmax=itmax, compensated=compensated, custom_init=custom_init,
                       precision=precision)
    return _out(r.reshape(out_shape), was_np)


# ---------------------------------------------------------------------------
# critical curves and caustics
# ---------------------------------------------------------------------------

def critical_and_caustic_curves(npts=200, nlenses=2, roots_itmax=2000, device=None, **params):
    """(critical_curves, caustic_curves), each [2*nlenses, npts] complex, one
    continuous curve per row, in the centre-of-mass frame
    (point_source.py:1582-1649).  NumPy out, or CUDA tensors on `device`."""
    dev = torch.device(device) if device is not None else None
    if dev is None and not torch.cuda.is_available():
        raise L.CausticsError("caustics_gb300 needs a CUDA device (no CPU fallback)")
    dev = dev or torch.device("cuda", torch.cuda.current_device())
    if nlenses == 1:  # the Einstein ring and a point caustic
        phi = torch.linspace(-math.pi, math.pi, npts, dtype=torch.float64, device=dev)
        zcr, zca = torch.exp(-1j * phi)[None, :], torch.zeros((1, npts), dtype=torch.complex128, device=dev)
    else:
        lens = L.lens_params(nlenses, params)
        deg = 2 * nlenses
        zcr = torch.empty((deg, npts), dtype=torch.complex128, device=dev)
        zca = torch.empty((deg, npts), dtype=torch.complex128, device=dev)
        nbytes = int(L.lib().cgb_critical_curves_workspace_bytes(npts, nlenses))
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        st = torch.zeros(1, dtype=torch.int32, device=dev)
        with torch.cuda.device(dev):
            L.check(L.lib().cgb_critical_and_caustic_curves(int(npts), lens, int(roots_itmax), _ptr(zcr), _ptr(zca),
                                                            _ptr(st), _ptr(ws), nbytes, _stream()),
                    "cgb_critical_and_caustic_curves")
    if device is not None:
        return zcr, zca
    return zcr.cpu().numpy(), zca.cpu().numpy()


# ---------------------------------------------------------------------------
# lens equation helpers (elementwise, on device)
# ---------------------------------------------------------------------------

def _lens_geometry(nlenses, params):
    if nlenses == 1:
        return [0.0 + 0.0j], [1.0], 0.0
    if nlenses == 2:
        if "a" in params:
            a, e1 = params["a"], params["e1"]
            return [a, -a], [e1, 1.0 - e1], 0.0
        s, q = params["s"], params["q"]
        a = 0.5 * s
        e1 = 1.0 / (1.0 + q)
        return [a, -a], [e1, 1.0 - e1], a * (1 - q) / (1 + q)
    if nlenses == 3:
        if "a" in params:
            a, r3, e1, e2 = params["a"], params["r3"], params["e1"], params["e2"]
            return [a, -a, complex(r3)], [e1, e2, 1.0 - e1 - e2], 0.0
        s, q, q3, r3, psi = (params[k] for k in ("s", "q", "q3", "r3", "psi"))
        a = 0.5 * s
        e1 = q / (1.0 + q + q3)
        e2 = q * e1
        return [a, -a, r3 * complex(math.cos(psi), math.sin(psi))], [e1, e2, 1.0 - e1 - e2], a * (1 - q) / (1 + q)
    raise ValueError("`nlenses` has to be set to be <= 3.")


def lens_polynomial(w, nlenses=2, **params):
    """Coefficients complex128 [..., nlenses^2 + 2], low -> high, of the
    lens-equation polynomial of each source position w (the frame of
    mag_point_source, shifted by x_cm): the reference's _poly_coeffs_binary /
    _poly_coeffs_triple (point_source.py:17-86, 89-1479; highest order first
    there) in product form, on the GPU (cgb_lens_polynomial)."""
    wt, was_np = _to_device(w, torch.complex128)
    wf = wt.reshape(-1).contiguous()
    deg = nlenses * nlenses + 1
    c = torch.empty((wf.numel(), deg + 1), dtype=torch.complex128, device=wf.device)
    with torch.cuda.device(wf.device):
        L.check(L.lib().cgb_lens_polynomial(_ptr(wf), _ptr(c), wf.numel(), L.lens_params(nlenses, params), _stream()),
                "cgb_lens_polynomial")
    return _out(c.reshape(tuple(wt.shape) + (deg + 1,)), was_np)


def lens_eq(z, nlenses=2, **params):
    """w = z - sum_j eps_j / (conj(z) - conj(r_j)) with the reference's
    (a, e1[, e2, r3]) parameters (point_source.py:1536-1556)."""
    zt, was_np = _to_device(z, torch.complex128)
    r, eps, _ = _lens_geometry(nlenses, params)
    zb = torch.conj(zt)
    w = zt.clone()
    for rj, ej in zip(r, eps):
        w = w - ej / (zb - complex(rj).conjugate())
    return _out(w, was_np)


def lens_eq_det_jac(z, nlenses=2, **params):
    """point_source.py:1558-1580."""
    zt, was_np = _to_device(z, torch.complex128)
    r, eps, _ = _lens_geometry(nlenses, params)
    zb = torch.conj(zt)
    s = torch.zeros_like(zt)
    for rj, ej in zip(r, eps):
        s = s + ej / (zb - complex(rj).conjugate()) ** 2
    return _out(1.0 - torch.abs(s) ** 2, was_np)


# ---------------------------------------------------------------------------
# magnifications
# ---------------------------------------------------------------------------

def mag_point_source(w, nlenses=2, roots_itmax=2500, roots_compensated=False, precision=None, return_status=False,
                     return_images=False, **params):
    """Point-source magnification (point_source.py:1762-1830)."""
    wt, was_np = _to_device(w, torch.complex128)
    shape = wt.shape
    wf = wt.reshape(-1).contiguous()
    n = wf.numel()
    mag = torch.empty(n, dtype=torch.float64, device=wf.device)
    st = torch.zeros(n, dtype=torch.int32, device=wf.device)
    deg = nlenses * nlenses + 1
    imgs = torch.empty((n, deg), dtype=torch.complex128, device=wf.device) if return_images else None
    msk = torch.empty(n, dtype=torch.int32, device=wf.device) if return_images else None
    prec = _precision(precision) if precision else (L.PREC_FP64_COMP if roots_compensated else L.PREC_FP64)
    with torch.cuda.device(wf.device):
        L.check(L.lib().cgb_mag_point_source(_ptr(wf), _ptr(mag), _ptr(imgs), _ptr(msk), n,
                                             L.lens_params(nlenses, params), int(roots_itmax), prec, _ptr(st),
                                             _stream()), "cgb_mag_point_source")
    out = [_out(mag.reshape(shape), was_np)]
    if return_images:
        out += [_out(imgs.reshape(tuple(shape) + (deg,)), was_np), _out(msk.reshape(shape), was_np)]
    if return_status:
        out.append(_out(st.reshape(shape), was_np))
    return out[0] if len(out) == 1 else tuple(out)


_LABELLING = {"reference": 0, "nearest": 1}


_TRIPLE_ROUTING = {"contour": 0, "reference": 1, "corrected": 2}


def _es_options(npts_limb, limb_darkening, u1, npts_ld, roots_itmax, precision, grid=0, queue_chunk=1, ld_group=1,
                grad_fp64_above=0.0, labelling="reference", triple_routing="contour", cta_threads=0, point_lanes=0):
    if labelling not in _LABELLING:
        raise ValueError(f"labelling must be one of {sorted(_LABELLING)}")
    if triple_routing not in _TRIPLE_ROUTING:
        raise ValueError(f"triple_routing must be one of {sorted(_TRIPLE_ROUTING)}")
    return L.EsOptions(int(npts_limb), int(bool(limb_darkening)), float(u1), int(npts_ld), int(roots_itmax),
                       _precision(precision or "fp64"), int(grid), int(queue_chunk), int(ld_group),
                       _LABELLING[labelling], float(grad_fp64_above), _TRIPLE_ROUTING[triple_routing],
                       int(cta_threads), int(point_lanes))


def _es_workspace(n, device):
    """Scratch of the single-evaluation *_ws entry points: one first-limb-point
    row order (8 bytes) per source position."""
    return torch.empty(max(n, 1), dtype=torch.int64, device=device)


def mag_extended_source(w0, rho, nlenses=2, npts_limb=150, limb_darkening=False, u1=0.0, npts_ld=100,
                        roots_itmax=2500, roots_compensated=False, precision=None, return_status=False, grid=0,
                        labelling="reference", **params):
    """Extended-source magnification (extended_source.py:741-904).  w0 may be a
    scalar (as in the reference) or an array of source centres (batched).
    labelling: "reference" reproduces the reference's limb image row order
    exactly; "nearest" matches roots by distance everywhere (faster)."""
    scalar = np.ndim(w0) == 0 and not isinstance(w0, torch.Tensor)
    wt, was_np = _to_device(np.atleast_1d(w0) if scalar else w0, torch.complex128)
    shape = wt.shape
    wf = wt.reshape(-1).contiguous()
    n = wf.numel()
    mag = torch.empty(n, dtype=torch.float64, device=wf.device)
    st = torch.zeros(n, dtype=torch.int32, device=wf.device)
    opts = _es_options(npts_limb, limb_darkening, u1, npts_ld, roots_itmax, precision, grid, labelling=labelling)
    ws = _es_workspace(n, wf.device)
    with torch.cuda.device(wf.device):
        L.check(L.lib().cgb_mag_extended_source_ws(_ptr(wf), _ptr(mag), n, float(rho), L.lens_params(nlenses, params),
                                                   opts, _ptr(st), _ptr(ws), ws.numel() * 8, _stream()),
                "cgb_mag_extended_source_ws")
    if scalar:
        m = float(mag[0].item())
        return (m, int(st[0].item())) if return_status else m
    out = _out(mag.reshape(shape), was_np)
    return (out, _out(st.reshape(shape), was_np)) if return_status else out


def mag(w_points, rho, nlenses=2, npts_limb=200, limb_darkening=False, u1=0.0, npts_ld=100, roots_itmax=2500,
        roots_compensated=False, precision=None, return_route=False, return_status=False, grid=0,
        labelling="reference", triple_routing="contour", **params):
    """Light curve: hexadecapole where the reference's tests accept it, contour
    integration elsewhere (lightcurve.py:99-254).  Triple lenses
    (triple_routing): "contour" integrates every point, as the reference's mag()
    (lightcurve.py:226-227); "reference" routes by the reference's triple
    hexadecapole and triple proximity test as written (lightcurve.py:37-46,
    third-lens terms at -r3), which accepts points where the hexadecapole is
    tens of percent off; "corrected" uses the same test with the third lens at
    r3, where the lens equation puts it."""
    wt, was_np = _to_device(w_points, torch.complex128)
    shape = wt.shape
    wf = wt.reshape(-1).contiguous()
    n = wf.numel()
    out = torch.empty(n, dtype=torch.float64, device=wf.device)
    route = torch.empty(n, dtype=torch.uint8, device=wf.device)
    st = torch.zeros(n, dtype=torch.int32, device=wf.device)
    opts = _es_options(npts_limb, limb_darkening, u1, npts_ld, roots_itmax, precision, grid, labelling=labelling,
                       triple_routing=triple_routing)
    ws = _es_workspace(n, wf.device)
    with torch.cuda.device(wf.device):
        L.check(L.lib().cgb_mag_ws(_ptr(wf), _ptr(out), _ptr(route), n, float(rho), L.lens_params(nlenses, params),
                                   opts, _ptr(st), _ptr(ws), ws.numel() * 8, _stream()), "cgb_mag_ws")
    res = [_out(out.reshape(shape), was_np)]
    if return_route:
        res.append(_out(route.reshape(shape).bool(), was_np))
    if return_status:
        res.append(_out(st.reshape(shape), was_np))
    return res[0] if len(res) == 1 else tuple(res)


# ---------------------------------------------------------------------------
# batched light curves and their vector-Jacobian product
# ---------------------------------------------------------------------------

CURVE_FIELDS = ("s", "q", "rho", "u1", "u0", "alpha", "t0", "tE")
CURVE_FIELDS_TRIPLE = ("s", "q", "q3", "r3", "psi", "rho", "u1", "u0", "alpha", "t0", "tE")


def _batched_args(offsets, t, curves, triple=False):
    off, _ = _to_device(offsets, torch.int64)
    tt, _ = _to_device(t, torch.float64)
    cv, _ = _to_device(curves, torch.float64)
    if not triple and (cv.ndim != 2 or cv.shape[1] != 8):
        raise ValueError("curves must have shape [ncurves, 8]: " + ", ".join(CURVE_FIELDS) +
                         " (triple lenses: [ncurves, 11]: " + ", ".join(CURVE_FIELDS_TRIPLE) + ")")
    if triple and (cv.ndim != 2 or cv.shape[1] != 11):
        raise ValueError("triple-lens curves must have shape [ncurves, 11]: " + ", ".join(CURVE_FIELDS_TRIPLE))
    if off.numel() != cv.shape[0] + 1:
        raise ValueError("offsets must have ncurves + 1 entries")
    return off.contiguous(), tt.contiguous(), cv.contiguous()


def _workspace(n, device, vjp=False, triple=False):
    lib = L.lib()
    nbytes = int(lib.cgb_mag_lc_batched_workspace_bytes(n) if not vjp else
                 (lib.cgb_mag_lc_batched_triple_vjp_workspace_bytes(n) if triple else
                  lib.cgb_mag_lc_batched_vjp_workspace_bytes(n)))
    return torch.empty(max(nbytes, 16), dtype=torch.uint8, device=device), nbytes


def mag_lc_batched(offsets, t, curves, npts_limb=200, limb_darkening=False, npts_ld=100, roots_itmax=2500,
                   precision="mixed", grid=0, queue_chunk=1, ld_group=1, return_route=False, return_status=False,
                   out=None, labelling="reference", cta_threads=0, point_lanes=0, triple_routing="contour"):
    """mag() for many light curves of uneven lengths in one pass.

    offsets: int64 [ncurves+1]; t: float64 [npoints]; curves: float64
    [ncurves, 8] = (s, q, rho, u1, u0, alpha, t0, tE) per binary-lens curve, or
    [ncurves, 11] = (s, q, q3, r3, psi, rho, u1, u0, alpha, t0, tE) per
    triple-lens curve (every point through the contour integral, as the
    reference's mag()); the source on the rectilinear trajectory.  Per-curve u1
    is used when limb_darkening.  grid, queue_chunk, ld_group, cta_threads,
    point_lanes: launch shape (autotune.tune)."""
    triple = np.ndim(curves) == 2 and np.shape(curves)[1] == 11
    off, tt, cv = _batched_args(offsets, t, curves, triple)
    n = tt.numel()
    dev = tt.device
    if out is None:
        mag_out = torch.empty(n, dtype=torch.float64, device=dev)
        route = torch.empty(n, dtype=torch.uint8, device=dev)
        st = torch.zeros(n, dtype=torch.int32, device=dev)
        ws, nbytes = _workspace(n, dev)
    else:  # caller-owned buffers (fixed-shape / graph-captured use)
        mag_out, route, st, ws = out
        nbytes = ws.numel()
    opts = _es_options(npts_limb, limb_darkening, 0.0, npts_ld, roots_itmax, precision, grid, queue_chunk, ld_group,
                       labelling=labelling, cta_threads=cta_threads, point_lanes=point_lanes,
                       triple_routing=triple_routing)
    fn = "cgb_mag_lc_batched_triple" if triple else "cgb_mag_lc_batched"
    with torch.cuda.device(dev):
        L.check(getattr(L.lib(), fn)(_ptr(off), _ptr(tt), _ptr(cv), cv.shape[0], n, _ptr(mag_out), _ptr(route),
                                     _ptr(st), opts, _ptr(ws), nbytes, _stream()), fn)
    res = [mag_out]
    if return_route:
        res.append(route.bool())
    if return_status:
        res.append(st)
    return res[0] if len(res) == 1 else tuple(res)


def mag_lc_batched_vjp(offsets, t, curves, cot, npts_limb=200, limb_darkening=False, npts_ld=100, roots_itmax=2500,
                       precision="mixed", grid=0, queue_chunk=1, ld_group=1, grad_fp64_above=0.0,
                       labelling="reference", cta_threads=0, point_lanes=0):
    """(grad [ncurves, 8 or 11], mag [npoints]): grad[c] = sum_i cot[i] d mag_i /
    d curves[c], for binary-lens curves [ncurves, 8] or triple-lens curves
    [ncurves, 11] (the columns of mag_lc_batched).  point_lanes is accepted for
    symmetry with mag_lc_batched; the adjoint's per-point pass takes one thread
    per point."""
    triple = np.ndim(curves) == 2 and np.shape(curves)[1] == 11
    off, tt, cv = _batched_args(offsets, t, curves, triple)
    ct, _ = _to_device(cot, torch.float64)
    n = tt.numel()
    dev = tt.device
    mag_out = torch.empty(n, dtype=torch.float64, device=dev)
    route = torch.empty(n, dtype=torch.uint8, device=dev)
    grad = torch.empty((cv.shape[0], cv.shape[1]), dtype=torch.float64, device=dev)
    ws, nbytes = _workspace(n, dev, vjp=True, triple=triple)
    opts = _es_options(npts_limb, limb_darkening, 0.0, npts_ld, roots_itmax, precision, grid, queue_chunk, ld_group,
                       grad_fp64_above, labelling, cta_threads=cta_threads)
    fn = "cgb_mag_lc_batched_triple_vjp" if triple else "cgb_mag_lc_batched_vjp"
    with torch.cuda.device(dev):
        L.check(getattr(L.lib(), fn)(_ptr(off), _ptr(tt), _ptr(cv), cv.shape[0], n, _ptr(ct.contiguous()),
                                     _ptr(grad), _ptr(mag_out), _ptr(route), None, opts, _ptr(ws), nbytes,
                                     _stream()), fn)
    return grad, mag_out


class LightCurveMagnification(torch.autograd.Function):
    """mag of batched light curves with the hand-written adjoint as backward:
    LightCurveMagnification.apply(curves [ncurves, 8], offsets, t, options dict)."""

    @staticmethod
    def forward(ctx, curves, offsets, t, options):
        ctx.save_for_backward(curves, offsets, t)
        ctx.options = dict(options)
        fwd = {k: v for k, v in ctx.options.items() if k != "grad_fp64_above"}
        return mag_lc_batched(offsets, t, curves.detach(), **fwd)

    @staticmethod
    def backward(ctx, gmag):
        curves, offsets, t = ctx.saved_tensors
        grad, _ = mag_lc_batched_vjp(offsets, t, curves.detach(), gmag.contiguous(), **ctx.options)
        return grad.to(curves.dtype), None, None, None


def mag_extended_source_grad(w0, rho, nlenses=2, npts_limb=150, limb_darkening=False, u1=0.0, npts_ld=100,
                             roots_itmax=2500, precision=None, grid=0, grad_fp64_above=0.0, labelling="reference",
                             **params):
    """(mag [n], grad [n, 6]) with grad = d mag / d(s, q, rho, u1, Re w0, Im w0)
    for binary lenses, grad [n, 9] with d mag / d(q3, r3, psi) appended for
    triple lenses: the hand-written adjoint of mag_extended_source.
    grad_fp64_above: in "mixed", contour points whose image tangents exceed it
    run the adjoint quadrature in FP64 (0 = default 6, < 0 = all)."""
    wt, was_np = _to_device(np.atleast_1d(w0) if np.ndim(w0) == 0 and not isinstance(w0, torch.Tensor) else w0,
                            torch.complex128)
    wf = wt.reshape(-1).contiguous()
    n = wf.numel()
    mag_out = torch.empty(n, dtype=torch.float64, device=wf.device)
    g = torch.empty((n, 6 if nlenses == 2 else 9), dtype=torch.float64, device=wf.device)
    opts = _es_options(npts_limb, limb_darkening, u1, npts_ld, roots_itmax, precision, grid,
                       grad_fp64_above=grad_fp64_above, labelling=labelling)
    ws = _es_workspace(n, wf.device)
    with torch.cuda.device(wf.device):
        L.check(L.lib().cgb_mag_extended_source_grad_ws(_ptr(wf), _ptr(mag_out), _ptr(g), n, float(rho),
                                                        L.lens_params(nlenses, params), opts, None, _ptr(ws),
                                                        ws.numel() * 8, _stream()),
                "cgb_mag_extended_source_grad_ws")
    return _out(mag_out, was_np), _out(g, was_np)


# ---------------------------------------------------------------------------
# annual-parallax trajectory
# ---------------------------------------------------------------------------

def project_onto_sky(vec, direction):
    """(east, north) components of 3-vectors vec [n, 3] (ICRS) on the plane of
    the sky perpendicular to `direction` (trajectory.py:45-80); host arithmetic."""
    d = np.asarray(direction, dtype=np.float64)
    d = d / np.linalg.norm(d)
    east = np.cross([0.0, 0.0, 1.0], d)
    north = np.cross(d, east)
    east, north = east / np.linalg.norm(east), north / np.linalg.norm(north)
    vec = np.asarray(vec, dtype=np.float64)
    return vec @ east, vec @ north


class _Parallax(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, traj, t):
        w, J = traj._launch(t, theta.detach(), True)
        ctx.save_for_backward(J)
        return w

    @staticmethod
    def backward(ctx, gw):
        (J,) = ctx.saved_tensors
        # real parameters, complex output: dL/dtheta_k = Re sum_i conj(gw_i) dw_i/dtheta_k
        return (torch.conj(gw)[:, None] * J).real.sum(0), None, None


class AnnualParallaxTrajectory:
    """Source trajectory with annual parallax (trajectory.py:12-157).  As in the
    reference, the constructor takes the observation times and the source's
    astropy SkyCoord and builds the projected Sun ephemeris on a 1-day grid with
    astropy; alternatively pass ephemeris=(t_jpl, s_e, s_n, s_e_dot, s_n_dot)
    computed elsewhere (e.g. project_onto_sky of the Earth's barycentric
    position and velocity, negated).  compute() runs on the GPU; with parameter
    tensors that require grad it is differentiable (torch autograd)."""

    def __init__(self, t, coords=None, ephemeris=None, device=None):
        if ephemeris is None:
            if coords is None:
                raise ValueError("pass coords (needs astropy) or a precomputed ephemeris")
            try:
                from astropy.coordinates import get_body_barycentric_posvel
                from astropy.time import Time
            except ImportError as e:
                raise L.CausticsError("building the ephemeris needs astropy; pass ephemeris= instead") from e
            t = np.asarray(t, dtype=np.float64)
            t_jpl = np.arange(t[0], t[-1] + 1, 1)
            pos, vel = get_body_barycentric_posvel("earth", Time(t_jpl + 2450000, format="jd", scale="tdb"))
            direction = np.array(coords.cartesian.xyz.value)
            s_e, s_n = project_onto_sky(-pos.xyz.value.T, direction)
            s_e_dot, s_n_dot = project_onto_sky(-vel.xyz.value.T, direction)
            ephemeris = (t_jpl, s_e, s_n, s_e_dot, s_n_dot)
        if not torch.cuda.is_available() and device is None:
            raise L.CausticsError("caustics_gb300 needs a CUDA device (no CPU fallback)")
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.ephemeris = [torch.as_tensor(np.asarray(a, dtype=np.float64), device=dev).contiguous() for a in ephemeris]
        self.device = dev

    def _launch(self, t, theta, jacobian):
        tt = t if isinstance(t, torch.Tensor) else torch.as_tensor(np.asarray(t, dtype=np.float64))
        tt = tt.to(self.device, torch.float64).contiguous()
        n = tt.numel()
        w = torch.empty(n, dtype=torch.complex128, device=self.device)
        J = torch.empty((n, 5), dtype=torch.complex128, device=self.device) if jacobian else None
        u0, t0, tE, piEE, piEN = (float(x) for x in theta)
        te, se, sn, sed, snd = self.ephemeris
        with torch.cuda.device(self.device):
            L.check(L.lib().cgb_parallax_trajectory(_ptr(te), _ptr(se), _ptr(sn), _ptr(sed), _ptr(snd), te.numel(),
                                                    _ptr(tt), n, u0, t0, tE, piEE, piEN, _ptr(w), _ptr(J), _stream()),
                    "cgb_parallax_trajectory")
        return w, J

    def compute(self, t, parametrization="cartesian", **params):
        """w(t) = east + i north (trajectory.py:122-157); params u0, t0, tE and
        piEE, piEN ("cartesian") or piE, psi ("polar")."""
        if parametrization == "polar":
            piEE = params["piE"] * (torch.sin(params["psi"]) if isinstance(params["psi"], torch.Tensor)
                                    else math.sin(params["psi"]))
            piEN = params["piE"] * (torch.cos(params["psi"]) if isinstance(params["psi"], torch.Tensor)
                                    else math.cos(params["psi"]))
        elif parametrization == "cartesian":
            piEE, piEN = params["piEE"], params["piEN"]
        else:
            raise ValueError("Invalid parametrization. Choose from 'polar' (piE, psi) or 'cartesian' (piEE, piEN).")
        vals = [params["u0"], params["t0"], params["tE"], piEE, piEN]
        if any(isinstance(v, torch.Tensor) and v.requires_grad for v in vals):
            theta = torch.stack([v.to(self.device, torch.float64).reshape(()) if isinstance(v, torch.Tensor)
                                 else torch.tensor(float(v), dtype=torch.float64, device=self.device) for v in vals])
            return _Parallax.apply(theta, self, t)
        w, _ = self._launch(t, [float(v) for v in vals], False)
        return w if isinstance(t, torch.Tensor) else w.cpu().numpy()

    def jacobian(self, t, u0, t0, tE, piEE, piEN):
        """(w [n], dw/d(u0, t0, tE, piEE, piEN) [n, 5]) on the device."""
        return self._launch(t, [u0, t0, tE, piEE, piEN], True)


class ExtendedSourceMagnification(torch.autograd.Function):
    """mag_extended_source as a function of the source centres w (complex
    tensor [n]) and params = (s, q, rho, u1) (float64 tensor [4]) for binary
    lenses; backward is the hand-written adjoint (mag_extended_source_grad).
    ExtendedSourceMagnification.apply(w, params, options)."""

    @staticmethod
    def forward(ctx, w, params, options):
        s, q, rho, u1 = (float(x) for x in params.detach().cpu())
        mag, g = mag_extended_source_grad(w.detach(), rho, u1=u1, s=s, q=q, **options)
        ctx.save_for_backward(g)
        return mag

    @staticmethod
    def backward(ctx, gmag):
        (g,) = ctx.saved_tensors
        gw = gmag * torch.complex(g[:, 4], g[:, 5])
        gp = (gmag[:, None] * g[:, :4]).sum(0)
        return gw, gp, None


# ---------------------------------------------------------------------------
# marginalised likelihood
# ---------------------------------------------------------------------------

def marginalized_log_likelihood_batched(offsets, A, fobs, C_inv, ll_cot=None, return_grad=False):
    """Per light curve c (points offsets[c] .. offsets[c+1]-1): (beta [n, 2],
    ll [n]) and, with return_grad, d ll / d A (times ll_cot[c] if given)."""
    off, _ = _to_device(offsets, torch.int64)
    a, was_np = _to_device(A, torch.float64)
    f, _ = _to_device(fobs, torch.float64)
    c, _ = _to_device(C_inv, torch.float64)
    n = off.numel() - 1
    dev = a.device
    beta = torch.empty((n, 2), dtype=torch.float64, device=dev)
    ll = torch.empty(n, dtype=torch.float64, device=dev)
    g = torch.empty_like(a) if return_grad else None
    lc = _to_device(ll_cot, torch.float64)[0] if ll_cot is not None else None
    with torch.cuda.device(dev):
        L.check(L.lib().cgb_marginalized_log_likelihood(_ptr(off), n, a.numel(), _ptr(a), _ptr(f), _ptr(c), _ptr(beta),
                                                        _ptr(ll), _ptr(g), _ptr(lc), _stream()),
                "cgb_marginalized_log_likelihood")
    out = (_out(beta, was_np), _out(ll, was_np))
    return out + (_out(g, was_np),) if return_grad else out


def marginalized_log_likelihood(A_list, fobs_list, C_inv_list, dense_covariance=False, Lam_sd=1e04):
    """(beta_list, ll): the log-likelihood summed over independent light curves,
    marginalised over (F_s, F_b) (linalg.py:10-94, diagonal covariance)."""
    if dense_covariance:
        raise NotImplementedError("dense_covariance=True: the reference's dense branch does not run "
                                  "(linalg.py:82-94 calls jnp.linals and an undefined M)")
    parts = [(_to_device(a, torch.float64), _to_device(f, torch.float64)[0], _to_device(c, torch.float64)[0])
             for a, f, c in zip(A_list, fobs_list, C_inv_list)]
    was_np = all(p[0][1] for p in parts)
    A = torch.cat([p[0][0].reshape(-1) for p in parts])
    lens = [p[0][0].numel() for p in parts]
    off = torch.as_tensor(np.concatenate([[0], np.cumsum(lens)]), dtype=torch.int64, device=A.device)
    beta, ll = marginalized_log_likelihood_batched(off, A, torch.cat([p[1].reshape(-1) for p in parts]),
                                                   torch.cat([p[2].reshape(-1) for p in parts]))
    betas = [_out(b, was_np) for b in beta]
    return betas, (float(ll.sum().item()) if was_np else ll.sum())


class LightCurveLogLikelihood(torch.autograd.Function):
    """Marginalised log-likelihood of batched light curves as a function of the
    curve parameters: LightCurveLogLikelihood.apply(curves [n, 8], offsets, t,
    fobs, C_inv, options) -> ll [n].  Backward: the likelihood's gradient with
    respect to the magnifications is the cotangent of the light-curve VJP."""

    @staticmethod
    def forward(ctx, curves, offsets, t, fobs, C_inv, options):
        ctx.options = dict(options)
        fwd = {k: v for k, v in ctx.options.items() if k != "grad_fp64_above"}
        mag = mag_lc_batched(offsets, t, curves.detach(), **fwd)
        _, ll = marginalized_log_likelihood_batched(offsets, mag, fobs, C_inv)
        ctx.save_for_backward(curves, offsets, t, fobs, C_inv, mag)
        return ll

    @staticmethod
    def backward(ctx, gll):
        curves, offsets, t, fobs, C_inv, mag = ctx.saved_tensors
        _, _, cot = marginalized_log_likelihood_batched(offsets, mag, fobs, C_inv, ll_cot=gll.contiguous(),
                                                        return_grad=True)
        grad, _ = mag_lc_batched_vjp(offsets, t, curves.detach(), cot, **ctx.options)
        return grad.to(curves.dtype), None, None, None, None, None


class BatchedLightCurves:
    """Fixed-shape batched light-curve evaluator.  Buffers (times, offsets,
    curve parameters, outputs and the work-queue workspace) are allocated once;
    the launch sequence of mag_lc_batched (queue reset, per-point pass,
    persistent contour kernel) is captured in a CUDA graph and replayed for new
    curve parameters; the launch shape comes from the autotuner."""

    def __init__(self, offsets, t, npts_limb=200, limb_darkening=False, npts_ld=100, roots_itmax=2500,
                 precision="mixed", tune=True, graph=True, curves_for_tuning=None, config=None, labelling="reference"):
        from . import autotune
        self.offsets, _ = _to_device(offsets, torch.int64)
        self.t, _ = _to_device(t, torch.float64)
        dev = self.t.device
        n = self.t.numel()
        self.curves = torch.zeros((self.offsets.numel() - 1, 8), dtype=torch.float64, device=dev)
        self.mag = torch.empty(n, dtype=torch.float64, device=dev)
        self.route = torch.empty(n, dtype=torch.uint8, device=dev)
        self.status = torch.zeros(n, dtype=torch.int32, device=dev)
        self.ws, _ = _workspace(n, dev)
        self.kw = dict(npts_limb=npts_limb, limb_darkening=limb_darkening, npts_ld=npts_ld, roots_itmax=roots_itmax,
                       precision=precision, labelling=labelling)
        if config is None:
            config = (autotune.tune(self.offsets, self.t, curves_for_tuning, **self.kw)
                      if tune and curves_for_tuning is not None else autotune.DEFAULT)
        self.config = dict(config)
        self.graph, self.graph_error = None, None
        if graph:
            if curves_for_tuning is not None:
                self.curves.copy_(torch.as_tensor(np.asarray(curves_for_tuning)) if not isinstance(
                    curves_for_tuning, torch.Tensor) else curves_for_tuning)
            side = torch.cuda.Stream(device=dev)
            side.wait_stream(torch.cuda.current_stream(dev))
            with torch.cuda.stream(side):
                self._launch()  # warm-up outside capture (sets kernel attributes)
            torch.cuda.current_stream(dev).wait_stream(side)
            self.graph = torch.cuda.CUDAGraph()
            try:
                with torch.cuda.graph(self.graph):
                    self._launch()
            except RuntimeError as e:  # capture refused: eager launches of the same kernels
                self.graph, self.graph_error = None, str(e)

    def _launch(self):
        return mag_lc_batched(self.offsets, self.t, self.curves, out=(self.mag, self.route, self.status, self.ws),
                              **self.kw, **self.config)

    def __call__(self, curves):
        """Magnifications for curve parameters [ncurves, 8]; returns the
        evaluator's output tensor (overwritten by the next call)."""
        self.curves.copy_(curves if isinstance(curves, torch.Tensor) else torch.as_tensor(np.asarray(curves)))
        if self.graph is not None:
            self.graph.replay()
        else:
            self._launch()
        return self.mag
