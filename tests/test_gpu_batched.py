"""Batched light curves (persistent device-queue kernel) and their
vector-Jacobian product, through the C ABI.

* values: identical to calling the single-curve mag() per curve, and within
  1e-4 of the oracle's mag() (lightcurve.py:99-254) on the same points;
* VJP: against central finite differences of sum_i cot_i mag_i (relative step
  1e-7, FP64 forward).  A finite difference is only used where it is stable
  (steps h and 2h agree to 1e-4): a discrete limb-refinement or linking decision
  that flips between +-h makes the function locally discontinuous;
* the torch.autograd.Function's backward is the same VJP.
"""
import numpy as np
import pytest
import torch

from oracle import caustics_oracle as O

pytestmark = pytest.mark.gpu
C = pytest.importorskip("caustics_gb300")
from caustics_gb300 import _lib as L  # noqa: E402


def draw_curves(ncurves, seed, nmin=20, nmax=60):
    """Parameters drawn as the reference-scale batched workload (s ~ logU[0.3,3],
    q ~ logU[1e-4,1], rho ~ logU[1e-3,1e-1], u0 ~ U[-0.3,0.3], alpha ~ U[0,2pi],
    u1 ~ U[0.2,0.8], tE ~ logU[5,100], t0 = 0), with short curves."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(nmin, nmax + 1, ncurves)
    cv = np.stack([10 ** rng.uniform(np.log10(0.3), np.log10(3), ncurves), 10 ** rng.uniform(-4, 0, ncurves),
                   10 ** rng.uniform(-3, -1, ncurves), rng.uniform(0.2, 0.8, ncurves), rng.uniform(-0.3, 0.3, ncurves),
                   rng.uniform(0, 2 * np.pi, ncurves), np.zeros(ncurves), 10 ** rng.uniform(np.log10(5), 2, ncurves)],
                  axis=1)
    offsets = np.concatenate([[0], np.cumsum(lens)])
    t = np.concatenate([np.sort(rng.uniform(-2 * te, 2 * te, n)) for te, n in zip(cv[:, 7], lens)])
    return offsets, t, cv


def traj(t, c):
    tau = (t - c[6]) / c[7]
    return (c[4] * np.cos(c[5]) + tau * np.sin(c[5])) + 1j * (-c[4] * np.sin(c[5]) + tau * np.cos(c[5]))


OPTS = dict(npts_limb=100, limb_darkening=True, npts_ld=40)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_matches_single_curve_calls(precision):
    off, t, cv = draw_curves(8, seed=2)
    m, route = C.mag_lc_batched(off, t, cv, precision=precision, return_route=True, **OPTS)
    m = m.cpu().numpy()
    for c in range(len(cv)):
        sl = slice(off[c], off[c + 1])
        w = traj(t[sl], cv[c])
        ref = C.mag(w, cv[c, 2], u1=cv[c, 3], s=cv[c, 0], q=cv[c, 1], precision=precision, **OPTS)
        # the batched pass evaluates the trajectory on the device, so source
        # positions differ from the host's by ~1e-16
        assert np.max(np.abs(m[sl] - ref) / ref) < (1e-12 if precision == "fp64" else 1e-10)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_first_point_order_kernel_matches_in_kernel_order(precision):
    """With a full workspace (16 + 16 n bytes) every first limb point is
    ordered by a kernel of its own ahead of the contour kernel; with the queue
    alone (16 + 8 n bytes) the contour kernel orders it itself.  The two give
    the same magnifications bit for bit."""
    off, t, cv = draw_curves(8, seed=21)
    n = len(t)
    full = C.mag_lc_batched(off, t, cv, precision=precision, **OPTS).cpu().numpy()
    dev = torch.device("cuda")
    out = (torch.empty(n, dtype=torch.float64, device=dev), torch.empty(n, dtype=torch.uint8, device=dev),
           torch.zeros(n, dtype=torch.int32, device=dev), torch.empty(16 + 8 * n, dtype=torch.uint8, device=dev))
    small = C.mag_lc_batched(off, t, cv, precision=precision, out=out, **OPTS).cpu().numpy()
    assert np.array_equal(full, small)


def test_batched_vs_oracle():
    off, t, cv = draw_curves(4, seed=5, nmin=6, nmax=10)
    m = C.mag_lc_batched(off, t, cv, precision="mixed", **OPTS).cpu().numpy()
    for c in range(len(cv)):
        sl = slice(off[c], off[c + 1])
        ref = O.mag(traj(t[sl], cv[c]), cv[c, 2], limb_darkening=True, u1=cv[c, 3], npts_limb=OPTS["npts_limb"],
                    npts_ld=OPTS["npts_ld"], s=cv[c, 0], q=cv[c, 1])
        assert np.max(np.abs(m[sl] - ref) / ref) < 1e-4


def test_empty_and_ragged():
    off = np.array([0, 0, 3, 3, 5])
    rng = np.random.default_rng(1)
    t = rng.uniform(-5, 5, 5)
    cv = np.tile([1.0, 0.1, 1e-2, 0.5, 0.1, 0.3, 0.0, 10.0], (4, 1))
    m = C.mag_lc_batched(off, t, cv, precision="mixed", **OPTS).cpu().numpy()
    assert m.shape == (5,) and np.all(np.isfinite(m)) and np.all(m >= 1.0)
    g, m2 = C.mag_lc_batched_vjp(off, t, cv, np.ones(5), precision="fp64", **OPTS)
    g = g.cpu().numpy()
    assert np.all(g[0] == 0) and np.all(g[2] == 0)  # curves without points


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_vjp_vs_central_differences(precision):
    off, t, cv = draw_curves(3, seed=3, nmin=8, nmax=12)
    rng = np.random.default_rng(4)
    cot = rng.normal(size=len(t))
    g, _ = C.mag_lc_batched_vjp(off, t, cv, cot, precision=precision, **OPTS)
    g = g.cpu().numpy()

    def f(cvv):
        return float(np.dot(cot, C.mag_lc_batched(off, t, cvv, precision="fp64", **OPTS).cpu().numpy()))

    checked = 0
    for c in range(len(cv)):
        for k in range(8):
            h = 1e-7 * max(abs(cv[c, k]), 1e-2 if k in (4, 5, 6) else 1e-3)
            est = []
            for step in (h, 2 * h):
                p, m = cv.copy(), cv.copy()
                p[c, k] += step
                m[c, k] -= step
                est.append((f(p) - f(m)) / (2 * step))
            if abs(est[0] - est[1]) > 1e-4 * max(abs(est[0]), 1e-6):
                continue  # a discrete decision flips within the step
            scale = max(abs(est[0]), 1e-3 * np.abs(cot).sum())
            assert abs(g[c, k] - est[0]) / scale < 1e-3, (c, k, g[c, k], est)
            checked += 1
    assert checked >= 12


def test_autograd_function_backward_is_the_vjp():
    off, t, cv = draw_curves(3, seed=7, nmin=8, nmax=12)
    curves = torch.tensor(cv, dtype=torch.float64, device="cuda", requires_grad=True)
    offs = torch.tensor(off, device="cuda")
    tt = torch.tensor(t, device="cuda")
    opts = dict(precision="mixed", **OPTS)
    m = C.LightCurveMagnification.apply(curves, offs, tt, opts)
    cot = torch.randn_like(m)
    (m * cot).sum().backward()
    g, _ = C.mag_lc_batched_vjp(offs, tt, curves.detach(), cot, **opts)
    # per-curve sums are accumulated with atomics, so two identical calls agree
    # only up to the summation order of point contributions
    assert torch.allclose(curves.grad, g, rtol=1e-9, atol=1e-12 * float(g.abs().max()))


def test_autotuned_graph_evaluator():
    """BatchedLightCurves: autotuned launch shape, launch sequence captured in a
    CUDA graph and replayed with new curve parameters; equals the eager call
    with the same launch shape, and the default shape within the reordering of
    the FP32 quadrature sums."""
    off, t, cv = draw_curves(6, seed=11)
    ev = C.BatchedLightCurves(off, t, curves_for_tuning=cv, precision="mixed", **OPTS)
    assert ev.graph is not None, ev.graph_error
    assert set(ev.config) == {"grid", "queue_chunk", "ld_group", "cta_threads", "point_lanes"}
    for seed in (11, 12):
        _, _, cv2 = draw_curves(6, seed=seed)
        m = ev(torch.as_tensor(cv2, device="cuda")).cpu().numpy()
        ref = C.mag_lc_batched(off, t, cv2, precision="mixed", **ev.config, **OPTS).cpu().numpy()
        assert np.max(np.abs(m - ref) / ref) < 1e-12
        ref = C.mag_lc_batched(off, t, cv2, precision="mixed", **OPTS).cpu().numpy()
        assert np.max(np.abs(m - ref) / ref) < 1e-6


@pytest.mark.parametrize("cfg", [dict(grid=7, queue_chunk=3, ld_group=4), dict(grid=1, queue_chunk=1, ld_group=8),
                                 dict(grid=0, queue_chunk=2, ld_group=2), dict(grid=0, cta_threads=128),
                                 dict(grid=5, cta_threads=64, ld_group=2), dict(point_lanes=8),
                                 dict(grid=0, cta_threads=128, point_lanes=8)])
def test_launch_shapes_agree(cfg):
    """Every launch shape the autotuner can pick gives the same magnifications."""
    off, t, cv = draw_curves(5, seed=13)
    ref = C.mag_lc_batched(off, t, cv, precision="fp64", **OPTS).cpu().numpy()
    m = C.mag_lc_batched(off, t, cv, precision="fp64", **cfg, **OPTS).cpu().numpy()
    assert np.max(np.abs(m - ref) / ref) < 1e-12
    g0, _ = C.mag_lc_batched_vjp(off, t, cv, np.ones(len(t)), precision="fp64", **OPTS)
    g1, _ = C.mag_lc_batched_vjp(off, t, cv, np.ones(len(t)), precision="fp64", **cfg, **OPTS)
    assert torch.allclose(g0, g1, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_point_lanes_group_solver(precision):
    """The per-point pass with a group of 8 lanes per polynomial (one lane per
    root) against one thread per polynomial: the same routing, hexadecapole
    magnifications equal to rounding, over curves whose points take both
    routes; the flags of the group solve are the thread solve's bits."""
    off, t, cv = draw_curves(12, seed=21)
    m1, r1, s1 = C.mag_lc_batched(off, t, cv, precision=precision, return_route=True, return_status=True, **OPTS)
    m8, r8, s8 = C.mag_lc_batched(off, t, cv, precision=precision, return_route=True, return_status=True,
                                  point_lanes=8, **OPTS)
    assert torch.equal(r1, r8)
    assert (~r1).sum().item() > 0 and r1.sum().item() > 0
    hex_ = ~r1
    assert torch.allclose(m8[hex_], m1[hex_], rtol=1e-11, atol=0)
    assert torch.allclose(m8[r1], m1[r1], rtol=1e-12, atol=0)
    assert not ((s8 | s1) & (L.ST_INVALID | L.ST_CAPACITY)).any()


def test_point_lanes_refused_values():
    off, t, cv = draw_curves(2, seed=3)
    with pytest.raises(L.CausticsError, match="point_lanes"):
        C.mag_lc_batched(off, t, cv, precision="fp64", point_lanes=4, **OPTS)


def draw_triple_curves(ncurves, seed, nmin=10, nmax=20):
    """Triple-lens curves: lenses drawn as the triple point-source workload (s,
    r3 ~ U[0.5, 2], q ~ logU[1e-4, 1], q3 ~ logU[1e-4, 1e-1], psi ~ U[0, 2pi]),
    sources and trajectories as the batched workload."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(nmin, nmax + 1, ncurves)
    cv = np.stack([rng.uniform(0.5, 2, ncurves), 10 ** rng.uniform(-4, 0, ncurves), 10 ** rng.uniform(-4, -1, ncurves),
                   rng.uniform(0.5, 2, ncurves), rng.uniform(0, 2 * np.pi, ncurves),
                   10 ** rng.uniform(-3, -1.5, ncurves), rng.uniform(0.2, 0.8, ncurves), rng.uniform(-0.3, 0.3, ncurves),
                   rng.uniform(0, 2 * np.pi, ncurves), np.zeros(ncurves), 10 ** rng.uniform(np.log10(5), 2, ncurves)],
                  axis=1)
    offsets = np.concatenate([[0], np.cumsum(lens)])
    t = np.concatenate([np.sort(rng.uniform(-1.0 * te, 1.0 * te, n)) for te, n in zip(cv[:, 10], lens)])
    return offsets, t, cv


def _masses(cv):
    e1 = cv[:, 1] / (1 + cv[:, 1] + cv[:, 2])
    return np.stack([e1, cv[:, 1] * e1, 1 - e1 - cv[:, 1] * e1], axis=1)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_triple_light_curves(precision):
    """Triple-lens light curves in one batched call equal the single-curve
    mag() of each curve (the same contour kernel; every point through the
    contour integral, as the reference's mag()).  The batched kernel forms the
    source position on the device, the single-curve call takes it from the
    host: the same to 1e-9 where every mass fraction is >= 1e-2; around a lens
    of mass fraction below 1e-2 FP64 fixes the clustered roots only to ~1e-8
    (sqrt of the rounding), so 1e-6 there.  Mixed precision there is compared
    with the single-curve FP64 result (which takes FP64 for such lenses from
    the start), within 1e-4."""
    off, t, cv = draw_triple_curves(6, seed=31)
    kw = dict(npts_limb=100, limb_darkening=True, npts_ld=40)
    m, route, st = C.mag_lc_batched(off, t, cv, precision=precision, return_route=True, return_status=True, **kw)
    m, route, st = m.cpu().numpy(), route.cpu().numpy(), st.cpu().numpy()
    assert route.all() and not np.any(st & (L.ST_INVALID | L.ST_CAPACITY))
    small = (_masses(cv) < 1e-2).any(axis=1)
    assert small.any() and (~small).any()
    for c in range(len(cv)):
        s, q, q3, r3, psi, rho, u1, u0, al, t0, te = cv[c]
        tau = (t[off[c]:off[c + 1]] - t0) / te
        w = (u0 * np.cos(al) + tau * np.sin(al)) + 1j * (-u0 * np.sin(al) + tau * np.cos(al))
        single = precision if (precision == "fp64" or not small[c]) else "fp64"
        ref = C.mag(w, rho, nlenses=3, s=s, q=q, q3=q3, r3=r3, psi=psi, u1=u1, precision=single, **kw)
        tol = 1e-4 if single != precision else (1e-6 if small[c] else 1e-9)
        assert np.max(np.abs(m[off[c]:off[c + 1]] - ref) / ref) < tol, (c, small[c])


def test_batched_triple_refusals_and_invalid_curves():
    off, t, cv = draw_triple_curves(3, seed=32)
    with pytest.raises(L.CausticsError, match="triple_routing"):
        C.mag_lc_batched(off, t, cv, precision="fp64", npts_limb=100, triple_routing="corrected")
    cv = cv.copy()
    cv[1, 5] = -1.0  # rho < 0: that curve's points are not evaluated
    m, st = C.mag_lc_batched(off, t, cv, precision="fp64", npts_limb=100, return_status=True)
    m, st = m.cpu().numpy(), st.cpu().numpy()
    bad = slice(off[1], off[2])
    assert np.all(np.isnan(m[bad])) and np.all(st[bad] == L.ST_INVALID)
    assert np.all(np.isfinite(m[off[0]:off[1]])) and np.all(np.isfinite(m[off[2]:]))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_triple_vjp(precision):
    """The batched VJP of triple-lens light curves, grad [ncurves, 11] in the
    order (s, q, q3, r3, psi, rho, u1, u0, alpha, t0, tE), against the
    single-evaluation adjoint of each point (d mu / d(s, q, rho, u1, Re w,
    Im w, q3, r3, psi), itself checked against central differences in
    test_gpu_adjoint.py) chained through the trajectory on the host."""
    off, t, cv = draw_triple_curves(4, seed=33, nmin=6, nmax=10)
    kw = dict(npts_limb=100, limb_darkening=True, npts_ld=40)
    cot = np.random.default_rng(4).normal(size=len(t))
    g, m = C.mag_lc_batched_vjp(off, t, cv, cot, precision=precision, **kw)
    g = g.cpu().numpy()
    assert g.shape == (len(cv), 11)
    g2, _ = C.mag_lc_batched_vjp(off, t, cv, cot, precision=precision, **kw)
    assert np.array_equal(g, g2.cpu().numpy())  # fixed-order sums
    for c in range(len(cv)):
        s, q, q3, r3, psi, rho, u1, u0, al, t0, te = cv[c]
        sl = slice(off[c], off[c + 1])
        tau = (t[sl] - t0) / te
        sa, ca = np.sin(al), np.cos(al)
        w = (u0 * ca + tau * sa) + 1j * (-u0 * sa + tau * ca)
        _, J = C.mag_extended_source_grad(w, rho, nlenses=3, s=s, q=q, q3=q3, r3=r3, psi=psi, u1=u1,
                                          precision=precision, **kw)
        J = np.asarray(J)
        jx, jy = J[:, 4], J[:, 5]
        cols = [J[:, 0], J[:, 1], J[:, 6], J[:, 7], J[:, 8], J[:, 2], J[:, 3], jx * ca - jy * sa,
                jx * (-u0 * sa + tau * ca) + jy * (-u0 * ca - tau * sa), -(jx * sa + jy * ca) / te,
                -tau * (jx * sa + jy * ca) / te]
        ref = cot[sl] @ np.stack(cols, axis=1)
        scale = np.abs(cot[sl]) @ np.abs(np.stack(cols, axis=1))
        assert np.all(np.abs(g[c] - ref) <= 1e-6 * scale + 1e-12), (c, g[c], ref)
