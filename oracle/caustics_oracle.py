"""ORACLE — test infrastructure only.

A CPU (NumPy, FP64) restatement of the magnification hot path of
fbartolic/caustics, used as the checker for the CUDA kernels.  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may import this
module; the product (``caustics_gb300``) never does.

Parity of this restatement is pinned against golden fixtures produced by the
reference itself (tests/golden/make_golden.py runs the reference's own Python
source on a NumPy stand-in for JAX, with its compiled C++ root solver), see
tests/test_oracle_golden.py.

Reference map (file:line in fbartolic/caustics):
  lens polynomial ........... src/caustics/point_source.py:17-86 (binary), 89-1479 (triple)
                               derived here by eliminating conj(z) from the lens equation
  root solver ............... lib/ehrlich_aberth/ehrlich_aberth.h (C restatement: oracle/ea_oracle.c)
  lens_eq / det J ........... src/caustics/point_source.py:1536-1580
  image filter .............. src/caustics/point_source.py:1652-1709 (|lens_eq(z) - w| < 1e-6)
  mag_point_source .......... src/caustics/point_source.py:1762-1830
  limb images ............... src/caustics/extended_source.py:56-153
  greedy image matching ..... src/caustics/utils.py:15-40, extended_source.py:34-53
  segments .................. src/caustics/extended_source.py:156-309
  segment merging ........... src/caustics/extended_source.py:312-727
  integrals ................. src/caustics/integrate.py:18-121, utils.py:89-100
  mag_extended_source ....... src/caustics/extended_source.py:741-904
  hexadecapole .............. src/caustics/multipole.py:8-244 (re-derived generically here)
  proximity / planet tests .. src/caustics/lightcurve.py:23-85
  mag ....................... src/caustics/lightcurve.py:99-254
  critical curves ........... src/caustics/point_source.py:1482-1534, 1582-1649
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from functools import lru_cache

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))

# ----------------------------------------------------------------------------
# C solver (oracle/ea_oracle.c)
# ----------------------------------------------------------------------------


@lru_cache(maxsize=1)
def _solver_lib():
    path = os.path.join(_HERE, "_build", "libea_oracle.so")
    src = os.path.join(_HERE, "ea_oracle.c")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE, "all"])
    lib = ctypes.CDLL(path)
    lib.oracle_ea_solve.restype = ctypes.c_int
    lib.oracle_ea_solve.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p]
    return lib


def ea_solve(coeffs_low_high, itmax=2500, compensated=False, roots_init=None, init_mode=1, return_iters=False):
    """Roots of polynomials given low->high (the reference's custom-call order).

    init_mode 1 reproduces the reference's real-valued initial guesses
    (lib/ehrlich_aberth/init_est.h:95); 0 uses complex guesses on the circle.
    """
    c = np.ascontiguousarray(coeffs_low_high, dtype=np.complex128)
    shp = c.shape
    deg = shp[-1] - 1
    c = c.reshape(-1, deg + 1)
    n = c.shape[0]
    roots = np.zeros((n, deg), dtype=np.complex128)
    iters = np.zeros(n, dtype=np.int32)
    ci = 0
    if roots_init is not None:
        ri = np.ascontiguousarray(np.asarray(roots_init, dtype=np.complex128).reshape(n, deg))
        ci = 1
    else:
        ri = np.zeros((1, deg), dtype=np.complex128)
    rc = _solver_lib().oracle_ea_solve(n, deg, int(itmax), int(bool(compensated)), ci, int(init_mode),
                                       c.ctypes.data, ri.ctypes.data, roots.ctypes.data, iters.ctypes.data)
    if rc != 0:
        raise ValueError("oracle_ea_solve rejected its arguments")
    roots = roots.reshape(shp[:-1] + (deg,))
    if return_iters:
        return roots, iters.reshape(shp[:-1])
    return roots


def poly_roots(coeffs, itmax=2000, compensated=False, custom_init=False, roots_init=None, init_mode=1):
    """Same contract as src/caustics/ehrlich_aberth_primitive.py:34-94 (coefficients highest order first)."""
    coeffs = np.asarray(coeffs, dtype=np.complex128)
    return ea_solve(coeffs[..., ::-1], itmax=itmax, compensated=compensated,
                    roots_init=roots_init if custom_init else None, init_mode=init_mode)


def roots_jvp(p, z, dp):
    """Implicit-function JVP of the roots (src/caustics/ehrlich_aberth_primitive.py:252-312):
    p, dp [M, deg+1] low->high, z [M, deg] -> dz_r = -sum_k z_r^k dp_k / p'(z_r)."""
    p, z, dp = (np.asarray(x, dtype=np.complex128) for x in (p, z, dp))
    deg = p.shape[1] - 1
    dfdz = np.stack([np.polyval(np.polyder(pi[::-1]), zi) for pi, zi in zip(p, z)])  # :292-293
    dfdp = z[..., None] ** np.arange(deg + 1)  # [M, deg, deg+1], :301
    return -np.einsum("mrk,mk->mr", dfdp, dp) / dfdz  # :304-307


# ----------------------------------------------------------------------------
# Lens configuration
# ----------------------------------------------------------------------------


class Lens:
    """Point lenses at positions r_j (complex) with mass fractions eps_j.

    Conventions of the reference (point_source.py:1798-1817): binary lenses at
    +a (mass e1) and -a (mass 1-e1), a = s/2, e1 = 1/(1+q); triple adds a third
    lens at r3*exp(i psi) with e1 = q/(1+q+q3), e2 = q*e1 (sic), e3 = 1-e1-e2.
    Source positions are shifted by x_cm = a(1-q)/(1+q) before solving.
    """

    def __init__(self, r, eps, x_cm=0.0):
        self.r = np.asarray(r, dtype=np.complex128)
        self.eps = np.asarray(eps, dtype=np.float64)
        self.x_cm = float(x_cm)

    @property
    def n(self):
        return len(self.r)

    @staticmethod
    def binary(s, q):
        a = 0.5 * s
        e1 = 1.0 / (1.0 + q)
        return Lens([a, -a], [e1, 1.0 - e1], a * (1 - q) / (1 + q))

    @staticmethod
    def binary_ae(a, e1):
        return Lens([a, -a], [e1, 1.0 - e1], 0.0)

    @staticmethod
    def triple(s, q, q3, r3, psi):
        a = 0.5 * s
        e1 = q / (1.0 + q + q3)
        e2 = q * e1
        return Lens([a, -a, r3 * np.exp(1j * psi)], [e1, e2, 1.0 - e1 - e2], a * (1 - q) / (1 + q))

    @staticmethod
    def triple_raw(a, r3, e1, e2):
        return Lens([a, -a, r3], [e1, e2, 1.0 - e1 - e2], 0.0)


def _pmul(p, q):
    """Product of polynomials stored low->high on the last axis (broadcasting)."""
    p, q = np.asarray(p), np.asarray(q)
    n, m = p.shape[-1], q.shape[-1]
    shape = np.broadcast_shapes(p.shape[:-1], q.shape[:-1]) + (n + m - 1,)
    out = np.zeros(shape, dtype=np.complex128)
    for i in range(n):
        out[..., i:i + m] += p[..., i:i + 1] * q
    return out


def _padd(p, q):
    n = max(p.shape[-1], q.shape[-1])
    pp = np.zeros(np.broadcast_shapes(p.shape[:-1], q.shape[:-1]) + (n,), dtype=np.complex128)
    pp[..., :p.shape[-1]] += p
    pp[..., :q.shape[-1]] += q
    return pp


def lens_polynomial(w, lens):
    """Coefficients (highest order first, like point_source.py:17-86/89-1479) of
    the degree n^2+1 polynomial whose roots contain the images of source w.

    With D(z) = prod_j (z - r_j), N(z) = sum_j eps_j prod_{k!=j} (z - r_k) and
    G_j(z) = (conj(w) - conj(r_j)) D(z) + N(z), substituting conj(z) = conj(w) +
    N/D into w = z - sum_j eps_j/(conj(z) - conj(r_j)) gives
        P(z) = (z - w) prod_j G_j - D sum_j eps_j prod_{k!=j} G_k.
    """
    w = np.asarray(w, dtype=np.complex128)
    wb = np.conj(w)[..., None]
    one = np.ones(1, dtype=np.complex128)
    D = one
    for rj in lens.r:
        D = _pmul(D, np.array([-rj, 1.0]))
    N = np.zeros(1, dtype=np.complex128)
    for j in range(lens.n):
        t = np.array([lens.eps[j]], dtype=np.complex128)
        for k in range(lens.n):
            if k != j:
                t = _pmul(t, np.array([-lens.r[k], 1.0]))
        N = _padd(N, t)
    G = [_padd((wb - np.conj(lens.r[j])) * D, np.broadcast_to(N, wb.shape[:-1] + N.shape)) for j in range(lens.n)]
    zw = np.concatenate([-w[..., None], np.ones_like(w)[..., None]], axis=-1)
    P = zw
    for g in G:
        P = _pmul(P, g)
    S = None
    for j in range(lens.n):
        t = lens.eps[j] * np.ones_like(G[0][..., :1])
        for k in range(lens.n):
            if k != j:
                t = _pmul(t, G[k])
        S = t if S is None else _padd(S, t)
    P = _padd(P, -_pmul(np.broadcast_to(D, S.shape[:-1] + D.shape), S))
    return P[..., ::-1]


def lens_eq(z, lens):
    """w = z - sum eps_j / (conj(z) - conj(r_j))  (point_source.py:1536-1556)."""
    zb = np.conj(z)
    w = np.array(z, dtype=np.complex128, copy=True)
    for rj, ej in zip(lens.r, lens.eps):
        w = w - ej / (zb - np.conj(rj))
    return w


def lens_eq_det_jac(z, lens):
    """det J = 1 - |sum eps_j / (conj(z) - conj(r_j))^2|^2  (point_source.py:1558-1580)."""
    zb = np.conj(z)
    s = 0
    for rj, ej in zip(lens.r, lens.eps):
        s = s + ej / (zb - np.conj(rj)) ** 2
    return 1.0 - np.abs(s) ** 2


def images_point_source(w, lens, itmax=2500, compensated=False, roots_init=None, init_mode=1):
    """Images of source positions w (already shifted by x_cm), image axis first
    (point_source.py:1652-1709)."""
    w = np.asarray(w, dtype=np.complex128)
    z = poly_roots(lens_polynomial(w, lens), itmax=itmax, compensated=compensated,
                   custom_init=roots_init is not None, roots_init=roots_init, init_mode=init_mode)
    z = np.moveaxis(z, -1, 0)
    mask = np.abs(lens_eq(z, lens) - w) < 1e-6
    return z, mask


def mag_point_source(w, nlenses=2, roots_itmax=2500, roots_compensated=False, init_mode=1, **params):
    """point_source.py:1762-1830."""
    lens = _lens_from_params(nlenses, params)
    w = np.asarray(w, dtype=np.complex128) + lens.x_cm
    z, mask = images_point_source(w, lens, itmax=roots_itmax, compensated=roots_compensated, init_mode=init_mode)
    det = lens_eq_det_jac(z, lens)
    return np.sum(mask / np.abs(det), axis=0)


def _lens_from_params(nlenses, params):
    if nlenses == 2:
        return Lens.binary(params["s"], params["q"])
    if nlenses == 3:
        return Lens.triple(params["s"], params["q"], params["q3"], params["r3"], params["psi"])
    raise ValueError("nlenses must be 2 or 3")


# ----------------------------------------------------------------------------
# Extended source: limb images, matching, segments, merging, integrals
# ----------------------------------------------------------------------------


def _jitter(shape, scale, salt):
    """Deterministic stand-in for the reference's PRNGKey(0) draws
    (extended_source.py:83-85, 146): root t of every warm start is moved by
    (+-scale/2, +-scale/2), signs from bits 0 and 1 of t; the CUDA kernels use
    the same pattern."""
    t = np.arange(shape[-1])
    re = np.where(t & 1, 0.5, -0.5) * scale
    im = np.where(t & 2, 0.5, -0.5) * scale
    return np.broadcast_to(re + 1j * im, shape)


def match_points(a, b):
    """Greedy nearest-neighbour assignment (utils.py:15-40): for each a_i in order
    take the closest b not yet taken.  Returns indices permuting b."""
    d = np.abs(b[None, :] - a[:, None])
    order = np.argsort(d, axis=1, kind="stable")
    taken = []
    for i in range(len(a)):
        for j in order[i]:
            if j not in taken:
                taken.append(j)
                break
    return np.array(taken, dtype=np.int64)


def images_of_source_limb(w0, rho, lens, npts=300, niter=10, itmax=2500, init_mode=1):
    """Ordered limb images (extended_source.py:56-153).  w0 is already shifted.

    Returns z (deg, L), mask (deg, L), parity (deg, L), theta (L,)."""
    deg = lens.n ** 2 + 1
    n0 = int(0.5 * npts)
    theta = np.concatenate([np.linspace(-np.pi, np.pi, n0 - 1, endpoint=False), [np.pi - 1e-8]])
    w = rho * np.exp(1j * theta) + w0
    coeffs = lens_polynomial(w, lens)[:, ::-1]
    z = np.zeros((len(theta), deg), dtype=np.complex128)
    # sequential warm start along the limb (point_source.py:1711-1759)
    z[0] = ea_solve(coeffs[0], itmax=itmax, init_mode=init_mode)
    for k in range(1, len(theta)):
        z[k] = ea_solve(coeffs[k], itmax=itmax, roots_init=z[k - 1])
    z = z.T
    mask = np.abs(lens_eq(z, lens) - w[None, :]) < 1e-6
    parity = np.sign(lens_eq_det_jac(z, lens))

    n_add = int(int(0.5 * npts) / niter)
    for _ in range(niter):
        dz = np.abs(z[:, 1:] - z[:, :-1])
        dz = np.where(mask[:, 1:] | mask[:, :-1], dz, 0.0)
        dmax = dz.max(axis=0)
        idx = np.argsort(dmax, kind="stable")[::-1][:n_add]
        th_new = 0.5 * (theta[idx] + theta[idx + 1])
        w_new = rho * np.exp(1j * th_new) + w0
        init = z[:, idx].T + _jitter((len(idx), deg), 1e-6, 0)
        z_new = ea_solve(lens_polynomial(w_new, lens)[:, ::-1], itmax=itmax, roots_init=init).T
        m_new = np.abs(lens_eq(z_new, lens) - w_new[None, :]) < 1e-6
        p_new = np.sign(lens_eq_det_jac(z_new, lens))
        theta = np.insert(theta, idx + 1, th_new)
        z = np.insert(z, idx + 1, z_new, axis=1)
        mask = np.insert(mask, idx + 1, m_new, axis=1)
        parity = np.insert(parity, idx + 1, p_new, axis=1)

    # exact duplicates get a tiny perturbation (extended_source.py:139-148)
    flat = z.reshape(-1)
    _, first = np.unique(flat, return_index=True)
    dup = np.ones(flat.shape, dtype=bool)
    dup[first] = False
    if dup.any():
        z = np.where(dup.reshape(z.shape), z + _jitter(z.shape, 1e-9, 1).real, z)

    # chained greedy matching along the limb (extended_source.py:34-53)
    L = z.shape[1]
    zp, mp_, pp = z.copy(), mask.copy(), parity.copy()
    carry = z[:, 0]
    for k in range(L):
        idc = match_points(carry, z[:, k])
        zp[:, k], mp_[:, k], pp[:, k] = z[idc, k], mask[idc, k], parity[idc, k]
        carry = zp[:, k]
    return zp, mp_, pp, theta


def split_segment(z, parity, mask, n_parts=5):
    """Split one image track into runs of real images of one parity without
    jumps > 0.1 (extended_source.py:156-216).  Returns (2*n_parts, 3, L) complex."""
    L = len(z)
    seg = np.stack([z, parity.astype(np.complex128), mask.astype(np.complex128)])
    dzz = z[1:] - z[:-1]
    jump = dzz.real ** 2 + dzz.imag ** 2 > 0.1 ** 2
    dpar = parity[1:].real - parity[:-1].real
    dmsk = mask[1:].real - mask[:-1].real
    change = np.concatenate([[mask[0] != 0], jump | (dpar != 0) | (dmsk != 0), [mask[-1] != 0]])
    dfull = np.concatenate([[1.0 if mask[0] != 0 else 0.0], dmsk, [-1.0 if mask[-1] != 0 else 0.0]])
    starts = np.flatnonzero(change & (dfull >= 0))[:2 * n_parts]
    ends = np.flatnonzero(change & (dfull <= 0))[:2 * n_parts]
    starts = np.pad(starts, (0, 2 * n_parts - len(starts)))
    ends = np.pad(ends, (0, 2 * n_parts - len(ends)))
    n = np.arange(L)
    out = np.zeros((2 * n_parts, 3, L), dtype=np.complex128)
    for k in range(2 * n_parts):
        l, r = starts[k], ends[k]
        if l == 0 and r == 0:
            continue
        out[k] = seg * ((n >= l) & (n < r))
    return out


def _first_nonzero(x):
    nz = np.flatnonzero(x != 0)
    return int(nz[0]) if len(nz) else 0


def _last_nonzero(x):
    nz = np.flatnonzero(x != 0)
    return int(nz[-1]) if len(nz) else 0


def _first_zero(x):
    nz = np.flatnonzero(x == 0)
    return int(nz[0]) if len(nz) else 0


def get_segments(z, mask, parity, nlenses=2):
    """Closed tracks and split open segments (extended_source.py:220-309)."""
    deg = z.shape[0]
    n_seg = 3 * (nlenses ** 2 + 1)
    zm = z * mask
    pm = parity * mask
    closed = (np.abs(zm[:, 0] - zm[:, -1]) < 1e-5) & np.all(mask, axis=1)
    seg = np.stack([zm, pm.astype(np.complex128), mask.astype(np.complex128)], axis=1)
    seg_closed = seg * closed[:, None, None]
    seg_open = seg * (~closed)[:, None, None]
    L = z.shape[1]
    if np.all(closed):
        opened = np.zeros((n_seg, 3, L), dtype=np.complex128)
    else:
        parts = np.concatenate([split_segment(s[0], s[1].real, s[2].real) for s in seg_open])
        cnt = np.sum(parts[:, 0] != 0, axis=1)
        parts = parts * (cnt >= 2)[:, None, None]
        order = np.argsort(np.any(np.abs(parts[:, 0, :]) > 0, axis=1), kind="stable")[::-1]
        parts = parts[order][:n_seg]
        opened = np.zeros_like(parts)
        for k in range(len(parts)):
            opened[k] = np.roll(parts[k], -_first_nonzero(np.abs(parts[k, 0])), axis=-1)
    return seg_closed[:, :2], opened[:, :2], bool(np.all(closed))


def _segment_head(x, t):
    if np.abs(x[1] - x[0]) > 1e-5 or t <= 1:
        return x[1], x[0]
    return x[2], x[1]


def _dyn2(x, s):
    s = min(max(int(s), 0), len(x) - 2)
    return x[s], x[s + 1]


def _segment_tail(x, t):
    if np.abs(x[t] - x[t - 1]) > 1e-5 or t <= 1:
        return _dyn2(x, t - 1)
    return _dyn2(x, t - 2)


def connection_condition(seg1, seg2, t1, t2, ctype, min_dist=1e-5, max_dist=1e-1, max_ang=60.0):
    """extended_source.py:324-442.  ctype 0 T-H, 1 H-T, 2 H-H, 3 T-T."""
    same = seg1[1, 0].real * seg2[1, 0].real > 0.0
    cond_par = same if ctype < 2 else (not same)
    x1, x2 = seg1[0], seg2[0]
    if ctype == 0:
        l1, l2 = _segment_tail(x1, t1), _segment_head(x2, t2)
    elif ctype == 1:
        l1, l2 = _segment_head(x1, t1), _segment_tail(x2, t2)
    elif ctype == 2:
        l1, l2 = _segment_head(x1, t1), _segment_head(x2, t2)
    else:
        l1, l2 = _segment_tail(x1, t1), _segment_tail(x2, t2)
    with np.errstate(all="ignore"):
        dist = np.abs(l1[1] - l2[1])
        v1 = (l1[1] - l1[0]) / np.abs(l1[1] - l1[0])
        v2 = (l2[1] - l2[0]) / np.abs(l2[1] - l2[0])
        ang = np.arccos(v1.real * v2.real + v1.imag * v2.imag)
        c1 = dist < max_dist
        c2 = (180.0 - np.rad2deg(ang)) < max_ang
        c3 = np.abs(l1[1] - l2[1]) < np.abs(l1[0] - l2[0])
    return bool(cond_par and ((c1 and c2 and c3) or dist < min_dist))


def _concat(first, second):
    return first + np.roll(second, _first_zero(np.abs(first[0])), axis=-1)


def merge_two_segments(seg1, seg2, t1, t2, ctype):
    """extended_source.py:445-492."""
    if ctype >= 2:
        s2 = seg2[:, ::-1]
        s2 = np.roll(s2, -(s2.shape[-1] - t2 - 1), axis=-1).copy()
        s2[1] = -s2[1]
        merged = _concat(s2, seg1) if ctype == 2 else _concat(seg1, s2)
    elif ctype == 0:
        merged = _concat(seg1, seg2)
    else:
        merged = _concat(seg2, seg1)
    return merged, t1 + t2 + 1


def _segment_length(seg, t):
    d = np.diff(seg[0])
    if 0 <= t < len(d):
        d[t] = 0.0
    return np.abs(d).sum()


def merge_open_segments(segments, max_contours=3, max_steps=20):
    """extended_source.py:495-667 (scan lengths max_steps, max_steps-2, ...)."""
    tails = np.array([_last_nonzero(s[0].real) for s in segments])
    L = segments.shape[-1]
    segs = np.concatenate([segments, np.zeros(segments.shape[:2] + (3 * L,), dtype=np.complex128)], axis=-1)
    merged_list = []
    for _ in range(max_contours):
        lengths = np.array([_segment_length(s, t) for s, t in zip(segs, tails)])
        order = np.argsort(np.where(lengths != 0, lengths, np.nan), kind="stable")
        segs, tails = segs[order], tails[order]
        act, tact = segs[0].copy(), int(tails[0])
        rest, rtails = segs[1:].copy(), tails[1:].copy()
        for _step in range(max_steps):
            if not np.any(rest[:, 0, 0] != 0):
                continue
            S = len(rest)
            tail_pts = rest[np.arange(S), 0, np.clip(rtails, 0, segs.shape[-1] - 1)]
            dists = np.stack([np.abs(act[0, tact] - rest[:, 0, 0]), np.abs(act[0, 0] - tail_pts),
                              np.abs(act[0, 0] - rest[:, 0, 0]), np.abs(act[0, tact] - tail_pts)])
            flat_order = np.argsort(dists.reshape(-1), kind="stable")[:4]
            cands = [divmod(int(f), S) for f in flat_order]
            succ = [connection_condition(act, rest[i], tact, int(rtails[i]), c) for c, i in cands]
            if any(succ):
                c, i = cands[succ.index(True)]
                act, tact = merge_two_segments(act, rest[i], tact, int(rtails[i]), c)
                rest[i] = 0.0
        merged_list.append(act)
        max_steps -= 2
        segs, tails = rest, rtails
    return np.stack(merged_list)


def contours_from_closed_segments(segments):
    p = segments[:, 1, 0].real
    c = segments[:, 0]
    return np.concatenate([c, c[:, :1]], axis=1), p


def contours_from_open_segments(segments, max_contours=3, max_steps=20):
    merged = merge_open_segments(segments, max_contours, max_steps)
    p = merged[:, 1, 0].real
    c = merged[:, 0].copy()
    for k in range(len(c)):
        t = _last_nonzero(c[k].real)
        if t + 1 < c.shape[1]:
            c[k, t + 1] = c[k, 0]
    return c, p


def _trapz_upto(y, x, t):
    """sum_{i<t} (y_i + y_{i+1})(x_{i+1} - x_i)/2  (= utils.py:89-100 for zero padding)."""
    t = int(t)
    return float(np.sum(0.5 * (y[:t] + y[1:t + 1]) * (x[1:t + 1] - x[:t])))


def integrate_unif(z, t):
    """integrate.py:23-27."""
    return _trapz_upto(0.5 * z.real, z.imag, t) + _trapz_upto(-0.5 * z.imag, z.real, t)


@lru_cache(maxsize=16)
def _leggauss(n):
    return np.polynomial.legendre.leggauss(n)


def brightness(z, rho, w0, u1, lens):
    """Linear limb-darkening profile in the Dominik (1998) form (integrate.py:29-44)."""
    r = np.abs(lens_eq(z, lens) - w0) / rho
    with np.errstate(all="ignore"):
        B = np.where(r <= 1.0, 1 + np.sqrt(np.maximum(1 - r ** 2, 0.0)), 1 - np.sqrt(np.maximum(1 - 1.0 / r ** 2, 0.0)))
    return 3.0 / (3.0 - u1) * (u1 * B + 1.0 - 2.0 * u1)


def _gl_line(a, b, rho, npts, f):
    """Integral of f from a to b split at b -/+ 2 rho (or a + |b-a|/2) with
    npts/2 + rest Gauss-Legendre nodes (integrate.py:49-78)."""
    absd = np.abs(b - a)
    split = np.where(b > a, b - 2 * rho, b + 2 * rho)
    split = np.where(0.5 * absd <= 2 * rho, a + 0.5 * absd, split)
    n1 = int(npts / 2)
    n2 = npts - n1
    tot = 0.0
    for lo, hi, n in ((a, split, n1), (split, b, n2)):
        x, wt = _leggauss(n)
        pts = 0.5 * (hi - lo) * x[:, None] + 0.5 * (hi + lo)
        tot = tot + np.sum(0.5 * (hi - lo) * f(pts) * wt[:, None], axis=0)
    return tot


def integrate_ld(z, t, w0, rho, u1, lens, npts=100):
    """integrate.py:47-121: Green's theorem with P = -1/2 int I dy, Q = 1/2 int I dx."""
    t = int(t)
    zc = z[:t + 1]
    z0 = z.sum() / (t + 1)
    xl, yl = zc.real, zc.imag
    P = -0.5 * _gl_line(z0.imag * np.ones_like(yl), yl, rho, npts,
                        lambda y: brightness(xl + 1j * y, rho, w0, u1, lens))
    Q = 0.5 * _gl_line(z0.real * np.ones_like(xl), xl, rho, npts,
                       lambda x: brightness(x + 1j * yl, rho, w0, u1, lens))
    return _trapz_upto(P, xl, t) + _trapz_upto(Q, yl, t)


def mag_extended_source(w0, rho, nlenses=2, npts_limb=150, limb_darkening=False, u1=0.0, npts_ld=100,
                        roots_itmax=2500, roots_compensated=False, init_mode=1, return_contours=False, **params):
    """extended_source.py:741-904."""
    lens = _lens_from_params(nlenses, params)
    w0 = complex(w0) + lens.x_cm
    z, mask, parity, _ = images_of_source_limb(w0, rho, lens, npts=npts_limb, itmax=roots_itmax,
                                               init_mode=init_mode)
    if limb_darkening:
        def integrate(c, t):
            return integrate_ld(c, t, w0, rho, u1, lens, npts=npts_ld)
    else:
        integrate = integrate_unif
    seg_closed, seg_open, all_closed = get_segments(z, mask, parity, nlenses)
    c1, p1 = contours_from_closed_segments(seg_closed)
    tot = sum(integrate(c, c1.shape[1] - 1) * p for c, p in zip(c1, p1))
    contours = [(c, c1.shape[1] - 1, p) for c, p in zip(c1, p1)]
    if not all_closed:
        c2, p2 = contours_from_open_segments(seg_open)
        for c, p in zip(c2, p2):
            t = _last_nonzero(c.real)
            tot += integrate(c, t) * p
            contours.append((c, t, p))
    mag = abs(tot) / (np.pi * rho ** 2)
    if return_contours:
        return mag, contours
    return mag


# ----------------------------------------------------------------------------
# Hexadecapole (multipole.py) — derived generically:
#   z(x, y) = z0 + sum a_kl x^k y^l / (k! l!),  w = z - conj(W1(z)),  W_k = W1^{(k-1)}
#   a_kl - conj(W2) conj(a_kl) = conj(Q_kl)  with Q_kl the order-(k+l) Taylor
#   coefficient of W1(z(x,y)) without its W2*a_kl term; image area A(rho) =
#   1/2 contour-integral Im(conj(z) dz) expanded in rho gives mu0, the quadrupole
#   and hexadecapole corrections.
# ----------------------------------------------------------------------------

_ORDER = 5


def _series_index():
    idx = {}
    for p in range(_ORDER + 1):
        for l in range(p + 1):
            idx[(p - l, l)] = len(idx)
    return idx


_SIDX = _series_index()


def _series_mul(A, B):
    """Truncated bivariate series product; coefficients stored as plain
    monomial coefficients c_kl of x^k y^l."""
    out = np.zeros_like(A)
    for (k1, l1), i1 in _SIDX.items():
        for (k2, l2), i2 in _SIDX.items():
            if k1 + l1 + k2 + l2 <= _ORDER:
                out[_SIDX[(k1 + k2, l1 + l2)]] += A[i1] * B[i2]
    return out


def hexadecapole_terms(W, rho, u1=0.0):
    """Per-image (mu0, delta_quad, delta_hex) from W = (W2..W6), each an array."""
    W = [np.asarray(x, dtype=np.complex128) for x in W]
    shape = W[0].shape
    nc = len(_SIDX)
    a = np.zeros((nc,) + shape, dtype=np.complex128)  # monomial coefficients of delta = z - z0
    W2c = np.conj(W[0])
    mu0 = 1.0 / (1.0 - np.abs(W[0]) ** 2)
    a[_SIDX[(1, 0)]] = mu0 * (1.0 + W2c)
    a[_SIDX[(0, 1)]] = mu0 * 1j * (1.0 - W2c)
    for p in range(2, _ORDER + 1):
        # Q at order p from sum_{m>=2} W_{m+1}/m! delta^m using orders < p of delta
        dpow = a.copy()
        qs = np.zeros_like(a)
        for m in range(2, p + 1):
            dpow = _series_mul(dpow, a)
            qs += W[m - 1] / math.factorial(m) * dpow
        for l in range(p + 1):
            k = p - l
            i = _SIDX[(k, l)]
            Q = qs[i] * math.factorial(k) * math.factorial(l)  # derivative-normalised
            akl = mu0 * (np.conj(Q) + W2c * Q)
            a[i] = akl / (math.factorial(k) * math.factorial(l))
    # area expansion: z(phi) = sum_p rho^p Z_p(phi), Z_p = sum_{k+l=p} a_kl c^k s^l
    mom = _trig_moments(2 * _ORDER + 2)
    A = {}
    for m in (2, 4, 6):
        acc = 0
        for p in range(1, m):
            q = m - p
            if p > _ORDER or q > _ORDER:
                continue
            # integral over phi of Im(conj(Z_p) dZ_q/dphi)
            for lp in range(p + 1):
                kp = p - lp
                for lq in range(q + 1):
                    kq = q - lq
                    # d/dphi c^kq s^lq = -kq c^(kq-1) s^(lq+1) + lq c^(kq+1) s^(lq-1)
                    t = 0.0
                    if kq > 0:
                        t = t - kq * mom[kp + kq - 1, lp + lq + 1]
                    if lq > 0:
                        t = t + lq * mom[kp + kq + 1, lp + lq - 1]
                    if t != 0.0:
                        acc = acc + np.conj(a[_SIDX[(kp, lp)]]) * a[_SIDX[(kq, lq)]] * t
        A[m] = 0.5 * np.imag(acc) / np.pi
    gamma = 2 * u1 / (3.0 - u1)
    mu_ps = A[2]
    dq = A[4] * (1.0 - gamma / 5.0) * rho ** 2
    dh = A[6] * (1.0 - 11.0 * gamma / 35.0) * rho ** 4
    return mu_ps, dq, dh


@lru_cache(maxsize=4)
def _trig_moments(n):
    """M[i, j] = integral_0^{2 pi} cos^i sin^j dphi (exact)."""
    M = np.zeros((n + 1, n + 1))
    for i in range(n + 1):
        for j in range(n + 1):
            if i % 2 or j % 2:
                continue
            # 2 * B((i+1)/2, (j+1)/2)
            M[i, j] = 2.0 * math.exp(math.lgamma((i + 1) / 2) + math.lgamma((j + 1) / 2) - math.lgamma((i + j + 2) / 2))
    return M


def mag_hexadecapole(z, mask, rho, lens, u1=0.0):
    """multipole.py:208-244: W_k = (-1)^(k-1) (k-1)! sum eps_j/(z - r_j)^k."""
    W = []
    for k in range(2, 7):
        s = 0
        for rj, ej in zip(lens.r, lens.eps):
            s = s + ej / (z - rj) ** k
        W.append((-1) ** (k - 1) * math.factorial(k - 1) * s)
    mu, dq, dh = hexadecapole_terms(W, rho, u1=u1)
    mu_multi = np.sum(mask * np.abs(mu + dq + dh), axis=0)
    dmu = np.sum(mask * np.abs(dq), axis=0) + np.sum(mask * np.abs(dh), axis=0)
    return mu_multi, dmu


def caustics_proximity_test(w, z, mask, rho, delta_mu, lens, c_m=1e-2, gamma=0.02, c_f=4.0, rho_min=1e-3):
    """lightcurve.py:23-75 (binary lens).  w is shifted."""
    (a, _), (e1, e2) = lens.r, lens.eps
    a = a.real
    f = lambda z: -e1 / (z - a) - e2 / (z + a)
    fp = lambda z: e1 / (z - a) ** 2 + e2 / (z + a) ** 2
    fpp = lambda z: 2 * (e1 / (a - z) ** 3 - e2 / (a + z) ** 3)
    zb = np.conj(z)
    zh = np.conj(w) - f(z)
    fp_z, fpp_z, fp_zb, fp_zh, fpp_zb = fp(z), fpp(z), fp(zb), fp(zh), fpp(zb)
    J = 1.0 - np.abs(fp_z * fp_zb)
    mu_cusp = 6 * np.imag(3 * fp_zb ** 3 * fpp_z ** 2) / J ** 5 * (rho + rho_min) ** 2
    mu_cusp = np.sum(np.abs(mu_cusp) * mask, axis=0)
    t_mc = gamma * mu_cusp + delta_mu < c_m
    Jh = 1 - np.abs(fp_z * fp_zh)
    with np.errstate(all="ignore"):
        fac = np.abs(J * Jh ** 2 / (Jh * fpp_zb * fp_z - np.conj(Jh) * fpp_z * fp_zb * fp_zh))
    t_f = 0.5 * np.sum(~mask * fac, axis=0) > c_f * (rho + rho_min)
    t_f = np.where(np.sum(~mask, axis=0) == 0, True, t_f)
    return t_f & t_mc


def caustics_proximity_test_triple(w, z, mask, rho, delta_mu, lens, as_written=True, c_m=1e-2, gamma=0.02, c_f=4.0,
                                   rho_min=1e-3):
    """The nlenses == 3 branch of lightcurve.py:23-75.  as_written: f, f', f''
    exactly as the reference writes them (lightcurve.py:37-46: third-lens terms
    at -r3 and f'' third term e3/(z+r3)^3); otherwise the third lens at r3 with
    f'' = -2 sum eps_j/(z - r_j)^3.  w is shifted."""
    a, e1, e2 = lens.r[0].real, lens.eps[0], lens.eps[1]
    e3 = 1 - e1 - e2
    r3 = -lens.r[2] if as_written else lens.r[2]
    c3 = 1.0 if as_written else -2.0
    f = lambda z: -e1 / (z - a) - e2 / (z + a) - e3 / (z - r3)
    fp = lambda z: e1 / (z - a) ** 2 + e2 / (z + a) ** 2 + e3 / (z - r3) ** 2
    fpp = lambda z: 2 * (e1 / (a - z) ** 3 - e2 / (a + z) ** 3) + c3 * e3 / (z - r3) ** 3
    zb = np.conj(z)
    zh = np.conj(w) - f(z)
    fp_z, fpp_z, fp_zb, fp_zh, fpp_zb = fp(z), fpp(z), fp(zb), fp(zh), fpp(zb)
    J = 1.0 - np.abs(fp_z * fp_zb)
    mu_cusp = 6 * np.imag(3 * fp_zb ** 3 * fpp_z ** 2) / J ** 5 * (rho + rho_min) ** 2
    mu_cusp = np.sum(np.abs(mu_cusp) * mask, axis=0)
    t_mc = gamma * mu_cusp + delta_mu < c_m
    Jh = 1 - np.abs(fp_z * fp_zh)
    with np.errstate(all="ignore"):
        fac = np.abs(J * Jh ** 2 / (Jh * fpp_zb * fp_z - np.conj(Jh) * fpp_z * fp_zb * fp_zh))
    t_f = 0.5 * np.sum(~mask * fac, axis=0) > c_f * (rho + rho_min)
    t_f = np.where(np.sum(~mask, axis=0) == 0, True, t_f)
    return t_f & t_mc


def planetary_caustic_test(w, rho, lens, c_p=2.0):
    """lightcurve.py:78-85, including q' = e1/(1-e1) (the inverse of q)."""
    a, e1 = lens.r[0].real, lens.eps[0]
    s = 2 * a
    q = e1 / (1 - e1)
    w_pc = -1 / s
    d_pc = 3 * np.sqrt(q) / s
    return (w_pc - w).real ** 2 + (w_pc - w).imag ** 2 > c_p * (rho ** 2 + d_pc ** 2)


def mag(w_points, rho, nlenses=2, npts_limb=200, limb_darkening=False, u1=0.0, npts_ld=100, roots_itmax=2500,
        roots_compensated=False, init_mode=1, return_route=False, **params):
    """lightcurve.py:99-254."""
    w_points = np.asarray(w_points, dtype=np.complex128)
    lens = _lens_from_params(nlenses, params)
    z, mask = images_point_source(w_points + lens.x_cm, lens, itmax=roots_itmax, compensated=roots_compensated,
                                  init_mode=init_mode)
    if nlenses == 2:
        mu_multi, dmu = mag_hexadecapole(z, mask, rho, lens)
        t1 = caustics_proximity_test(w_points + lens.x_cm, z, mask, rho, dmu, lens)
        t2 = planetary_caustic_test(w_points + lens.x_cm, rho, lens)
        test = (t1 & t2) if params["q"] < 0.01 else t1
    else:
        mu_multi = np.zeros(w_points.shape)
        test = np.zeros(w_points.shape, dtype=bool)
    out = np.array(mu_multi, dtype=np.float64)
    for i in np.flatnonzero(~test):
        out[i] = mag_extended_source(w_points[i], rho, nlenses=nlenses, npts_limb=npts_limb,
                                     limb_darkening=limb_darkening, u1=u1, npts_ld=npts_ld,
                                     roots_itmax=roots_itmax, roots_compensated=roots_compensated,
                                     init_mode=init_mode, **params)
    if return_route:
        return out, test
    return out


def trajectory(t, u0, alpha, t0, tE):
    """Rectilinear source trajectory (trajectory.py:152-155 with pi_E = 0)."""
    tau = (np.asarray(t) - t0) / tE
    return (u0 * np.cos(alpha) + tau * np.sin(alpha)) + 1j * (-u0 * np.sin(alpha) + tau * np.cos(alpha))


def critical_and_caustic_curves(npts=200, nlenses=2, init_mode=1, **params):
    """point_source.py:1582-1649: critical curves from the degree-2n polynomial
    sum eps_j/(z - r_j)^2 = exp(-i phi) (times the lens denominators), chained by
    greedy matching, mapped through the lens equation, shifted by x_cm."""
    phi = np.linspace(-np.pi, np.pi, npts)
    lens = _lens_from_params(nlenses, params)
    x = np.exp(-1j * phi)
    # prod_j (z - r_j)^2 * x - sum_j eps_j prod_{k != j} (z - r_k)^2 = 0
    sq = [np.array([rj ** 2, -2 * rj, 1.0], dtype=np.complex128) for rj in lens.r]
    prod_all = np.ones(1, dtype=np.complex128)
    for p in sq:
        prod_all = _pmul(prod_all, p)
    rest = np.zeros(1, dtype=np.complex128)
    for j in range(lens.n):
        t = np.array([lens.eps[j]], dtype=np.complex128)
        for k in range(lens.n):
            if k != j:
                t = _pmul(t, sq[k])
        rest = _padd(rest, t)
    coeffs = _padd(x[:, None] * prod_all[None, :], -np.broadcast_to(rest, (npts,) + rest.shape))
    z_cr = ea_solve(coeffs, itmax=2000, init_mode=init_mode)  # low->high already
    out = np.empty_like(z_cr)
    carry = z_cr[0]
    for k in range(npts):
        out[k] = z_cr[k][match_points(carry, z_cr[k])]
        carry = out[k]
    z_cr = out.T
    z_ca = lens_eq(z_cr, lens)
    return z_cr - lens.x_cm, z_ca - lens.x_cm


# ----------------------------------------------------------------------------
# Frozen-structure evaluation (for checking adjoints): the limb angle and the
# identity of every contour point are taken from a base evaluation; at perturbed
# parameters each point's image is re-solved and matched to its base image, and
# the same integrals are evaluated.  This is the smooth function that autodiff
# (the reference's, or a hand-written adjoint) differentiates: the limb
# refinement, matching and linking decisions are piecewise constant.
# ----------------------------------------------------------------------------


def contour_structure(w, rho, s, q, npts_limb, limb_darkening=False, u1=0.0, npts_ld=100):
    lens = Lens.binary(s, q)
    w0 = complex(w) + lens.x_cm
    _, contours = mag_extended_source(w, rho, npts_limb=npts_limb, limb_darkening=limb_darkening, u1=u1,
                                      npts_ld=npts_ld, s=s, q=q, return_contours=True)
    out = []
    for c, t, p in contours:
        zc = np.asarray(c[:t + 1])
        if not np.any(zc != 0):
            continue
        theta = np.angle(lens_eq(zc, lens) - w0)
        out.append((zc, theta, p))
    return out


def mag_es_frozen(structure, w, rho, s, q, limb_darkening=False, u1=0.0, npts_ld=100):
    lens = Lens.binary(s, q)
    w0 = complex(w) + lens.x_cm
    tot = 0.0
    for zbase, theta, p in structure:
        wl = w0 + rho * np.exp(1j * theta)
        roots = np.moveaxis(poly_roots(lens_polynomial(wl, lens), itmax=2500, init_mode=0), -1, 0)
        pick = np.argmin(np.abs(roots - zbase[None, :]), axis=0)
        z = roots[pick, np.arange(len(zbase))]
        t = len(z) - 1
        if limb_darkening:
            tot += p * integrate_ld(z, t, w0, rho, u1, lens, npts=npts_ld)
        else:
            tot += p * integrate_unif(z, t)
    return abs(tot) / (np.pi * rho ** 2)


def frozen_gradient(w, rho, s, q, npts_limb, limb_darkening=False, u1=0.0, npts_ld=100, rel=1e-6):
    """Central differences of the frozen-structure magnification with respect
    to (s, q, rho, u1, Re w, Im w)."""
    st = contour_structure(w, rho, s, q, npts_limb, limb_darkening, u1, npts_ld)
    base = dict(w=complex(w), rho=rho, s=s, q=q, u1=u1)
    g = np.zeros(6)
    for k, name in enumerate(("s", "q", "rho", "u1", "wx", "wy")):
        if name == "u1" and not limb_darkening:
            continue
        h = rel * (max(abs(base[name]), 1e-3) if name in base else 1.0)
        vals = []
        for sgn in (1, -1):
            p = dict(base)
            if name == "wx":
                p["w"] = base["w"] + sgn * h
            elif name == "wy":
                p["w"] = base["w"] + 1j * sgn * h
            else:
                p[name] = base[name] + sgn * h
            vals.append(mag_es_frozen(st, p["w"], p["rho"], p["s"], p["q"], limb_darkening, p["u1"], npts_ld))
        g[k] = (vals[0] - vals[1]) / (2 * h)
    return g


# ----------------------------------------------------------------------------
# Marginalised likelihood (linalg.py:10-94, diagonal covariance branch)
# ----------------------------------------------------------------------------


def marginalized_log_likelihood(A_list, fobs_list, C_inv_list):
    """Per light curve: weighted least squares for beta = (F_s, F_b) in
    f = F_s A + F_b (linalg.py:60-66), then
    ll = -chi2/2 + log det(2 pi Sigma)/2 with Sigma = (M^T C^-1 M)^-1 (:69-70).
    Returns (beta [n, 2], ll per curve); the reference returns the sum."""
    betas, lls = [], []
    for A, f, c in zip(A_list, fobs_list, C_inv_list):
        A, f, c = (np.asarray(x, dtype=np.float64) for x in (A, f, c))
        M = np.stack([A, np.ones_like(A)], axis=1)
        F = M.T @ (c[:, None] * M)
        Sig = np.linalg.inv(F)
        beta = Sig @ (M.T @ (c * f))
        r = f - M @ beta
        betas.append(beta)
        lls.append(-0.5 * np.sum(r * r * c) + 0.5 * np.log(np.linalg.det(2 * np.pi * Sig)))
    return np.array(betas), np.array(lls)


def marginalized_log_likelihood_grad(A, fobs, C_inv, beta, Sigma):
    """d ll / d A_i of one curve.  beta is the least-squares optimum, so chi2's
    dependence through beta drops out (envelope theorem):
    d ll / d A_i = c_i (r_i beta_0 - A_i Sigma_00 - Sigma_01)."""
    r = fobs - (beta[0] * A + beta[1])
    return C_inv * (r * beta[0] - A * Sigma[0, 0] - Sigma[0, 1])


# ----------------------------------------------------------------------------
# Annual-parallax trajectory (trajectory.py:106-157) and the sky projection of
# the Sun's position (trajectory.py:45-80)
# ----------------------------------------------------------------------------


def project_onto_sky(vec, direction):
    """East and north components of 3-vectors vec [n, 3] on the plane of the sky
    perpendicular to `direction` (ICRS), trajectory.py:45-80."""
    d = np.asarray(direction, dtype=np.float64)
    d = d / np.linalg.norm(d)
    east = np.cross([0.0, 0.0, 1.0], d)
    north = np.cross(d, east)
    east, north = east / np.linalg.norm(east), north / np.linalg.norm(north)
    vec = np.asarray(vec, dtype=np.float64)
    return vec @ east, vec @ north


def parallax_trajectory(t, t_jpl, s_e, s_n, s_e_dot, s_n_dot, u0, t0, tE, piEE, piEN):
    """Source position w(t) with annual parallax (trajectory.py:106-157,
    cartesian parametrisation): deviation of the Sun's projected position from
    rectilinear motion about t0, added with piE to the rectilinear trajectory of
    angle psi = atan2(piEE, piEN)."""
    t = np.asarray(t, dtype=np.float64)
    dse = np.interp(t, t_jpl, s_e) - np.interp(t0, t_jpl, s_e) - (t - t0) * np.interp(t0, t_jpl, s_e_dot)
    dsn = np.interp(t, t_jpl, s_n) - np.interp(t0, t_jpl, s_n) - (t - t0) * np.interp(t0, t_jpl, s_n_dot)
    psi, piE = np.arctan2(piEE, piEN), np.sqrt(piEN ** 2 + piEE ** 2)
    ue = u0 * np.cos(psi) + (t - t0) / tE * np.sin(psi) + piE * dse
    un = -u0 * np.sin(psi) + (t - t0) / tE * np.cos(psi) + piE * dsn
    return ue + 1j * un
