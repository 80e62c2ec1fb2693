"""GPU parity at the benchmark workloads' own sizes, against fixtures written
by the reference itself (tests/golden/make_golden.py):

* every point of the 2000-point limb-darkened light curve (s 1.1, q 5e-3,
  npts_limb 500);
* whole curves of the 4096-curve batched workload (seed 2, npts_limb 200,
  npts_ld 100) across the three mass-ratio ranges;
* the points of that workload that set a non-convergence or contour-linking
  status bit in a full run;
* gradients of four whole 1000-point curves of the 256-curve gradient
  workload (seed 3) against the reference's central differences, and the
  mixed-precision VJP of 64 of its curves against the FP64 VJP;
* triple-lens point source over all 1000 systems of the triple workload
  (seed 1), the mixed solver against FP64 at the full 10^6 positions;
* the triple hexadecapole and its proximity test (the reference's pieces,
  which its mag() never reaches for triple lenses).

Tolerances: FP64 1e-9 relative on magnifications (the contour is the
reference's own); mixed precision 1e-4 (the bound the path promises); routing
exact; gradients 1e-3 of the cotangent-weighted L1 scale (the reference's own
gradient tolerance, tests/test_extended_source.py:295-331); roots 1e-10
relative as sets unless a root's condition allows less; image counts exact
outside the band where a residual is within x30 of the 1e-6 filter threshold.
"""
import numpy as np
import pytest
import torch

from oracle import caustics_oracle as O

pytestmark = pytest.mark.gpu

C = pytest.importorskip("caustics_gb300")
from caustics_gb300 import _lib as L  # noqa: E402

BOUND = {"fp64": 1e-9, "mixed": 1e-4}
LC = dict(npts_limb=200, limb_darkening=True, npts_ld=100)


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)) / np.abs(np.asarray(b))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_light_curve_2000_points(G, precision):
    d = G("mag_lc_binary_ld_s1.1_q5e-3_2000pt")
    cv = d["curve"][None, :]
    off = np.array([0, len(d["t"])])
    m, route, st = C.mag_lc_batched(off, d["t"], cv, npts_limb=int(d["npts_limb"]), limb_darkening=True,
                                    npts_ld=int(d["npts_ld"]), precision=precision, return_route=True,
                                    return_status=True)
    m, route, st = m.cpu().numpy(), route.cpu().numpy(), st.cpu().numpy()
    assert np.array_equal(route, d["route"])
    assert rel(m, d["mag"]).max() < BOUND[precision]
    assert not np.any(st & (L.ST_CAPACITY | L.ST_INVALID))
    # the single-curve entry point gives the same light curve
    m1 = C.mag(d["w"], float(cv[0, 2]), npts_limb=int(d["npts_limb"]), limb_darkening=True, u1=float(cv[0, 3]),
               npts_ld=int(d["npts_ld"]), s=float(cv[0, 0]), q=float(cv[0, 1]), precision=precision)
    assert rel(m1, d["mag"]).max() < BOUND[precision]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_workload_curves(G, precision):
    d = G("mag_lc_batched_seed2_sample")
    m, route = C.mag_lc_batched(d["offsets"], d["t"], d["curves"], precision=precision, return_route=True, **LC)
    m, route = m.cpu().numpy(), route.cpu().numpy()
    assert np.array_equal(route, d["route"])
    assert rel(m, d["mag"]).max() < BOUND[precision]
    q = d["curves"][:, 1]
    assert (q < 1e-3).sum() >= 2 and ((q >= 1e-3) & (q < 1e-2)).sum() >= 2 and (q >= 1e-2).sum() >= 2


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_workload_flagged_points(G, precision):
    """The points of a full 4096-curve run whose evaluation set CGB_ST_NOCONV
    (mixed precision: a limb solve hit its iteration cap and took the FP64
    fallback) or CGB_ST_MERGE (the reference's segment linking leaves open
    segments), each as a curve of one point."""
    d = G("mag_lc_batched_seed2_flagged")
    n = len(d["t"])
    m, route, st = C.mag_lc_batched(np.arange(n + 1), d["t"], d["curves"], precision=precision, return_route=True,
                                    return_status=True, **LC)
    m, route, st = m.cpu().numpy(), route.cpu().numpy(), st.cpu().numpy()
    assert np.array_equal(route, d["route"])
    assert rel(m, d["mag"]).max() < BOUND[precision]
    assert np.any(st & L.ST_MERGE)  # the linking leaves open segments here, as in the reference
    assert m.min() < 1.0  # ... including a point the reference itself gives mu < 1


def _fd_noise(mag, cv):
    """Rounding noise of a central difference of the FP64 magnification at
    relative step 1e-7 (mu ~1e-13 relative over 2e-7 of the parameter's scale),
    per point and input (s, q, rho, u1, Re w, Im w), with a margin."""
    scale = np.array([cv[0], cv[1], cv[2], cv[3], cv[2], cv[2]])
    return 1e-5 * mag[:, None] / scale[None, :]


def _trusted(J1, J2, noise):
    """Points whose six central-difference derivatives agree between the two
    steps (the limb refinement, a discrete choice, did not change within +-h)."""
    return np.all(np.abs(J1 - J2) <= 2e-4 * np.maximum(np.abs(J1), np.abs(J2)) + noise, axis=1)


def _chain(J, t, cv, absolute=False):
    """d mag / d(s, q, rho, u1, u0, alpha, t0, tE) from the derivatives with
    respect to (s, q, rho, u1, Re w, Im w), w on the rectilinear trajectory
    (absolute: the same map on magnitudes, for error bounds)."""
    u0, al, t0, te = cv[4], cv[5], cv[6], cv[7]
    tau = (t - t0) / te
    sa, ca = np.sin(al), np.cos(al)
    cw = [(ca, -sa), (-u0 * sa + tau * ca, -u0 * ca - tau * sa), (-sa / te, -ca / te), (-tau * sa / te, -tau * ca / te)]
    jx, jy = J[:, 4], J[:, 5]
    f = np.abs if absolute else (lambda x: x)
    cols = [f(a) * jx + f(b) * jy for a, b in cw]
    return np.stack([J[:, 0], J[:, 1], J[:, 2], J[:, 3]] + cols, axis=1)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_vjp_full_length_curves_against_reference_differences(G, precision):
    """The VJP of four whole curves against the reference's per-point central
    differences (step 1e-7; points where the 1e-8 step disagrees, i.e. where a
    discrete choice changed within +-h, get a zero cotangent): 1e-3 of the
    cotangent-weighted L1 scale plus the differences' rounding noise."""
    d = G("vjp_seed3_fd")
    rng = np.random.default_rng(12)
    for c in d["curve_ids"]:
        t, cv, J = d[f"t{c}"], d[f"curve{c}"], d[f"jac{c}"]
        noise = _fd_noise(d[f"mag{c}"], cv)
        ok = _trusted(J[0], J[1], noise)
        assert ok.mean() > 0.85, (c, ok.mean())
        cot = np.where(ok, rng.normal(size=len(t)), 0.0)
        g, m = C.mag_lc_batched_vjp(np.array([0, len(t)]), t, cv[None, :], cot, precision=precision, **LC)
        g, m = g.cpu().numpy()[0], m.cpu().numpy()
        assert rel(m, d[f"mag{c}"]).max() < BOUND[precision]
        D = _chain(J[0], t, cv)
        ref = cot @ D
        tol = 1e-3 * (np.abs(cot) @ np.abs(D)) + np.abs(cot) @ _chain(noise, t, cv, absolute=True)
        assert np.all(np.abs(g - ref) <= tol), (c, g, ref, tol)


def test_mixed_vjp_against_fp64_gradient_workload():
    """Mixed-precision VJP against the FP64 VJP on the first 64 curves of the
    gradient workload (seed 3): per curve, |g_mixed - g_fp64| / |g_fp64| <=
    1e-4 (over all 256 curves: median 2e-7, p99 5e-5, largest 1.7e-4 on curve
    176, unchanged with every quadrature node in FP64, so that one comes from
    the forward pass's roots, not the adjoint).  Curve 7 (q 6e-4, rho 0.054)
    holds the evaluation where a quadrature node lies 1.3e-8 inside the limb:
    its FP32 1 - r^2 had the wrong sign and the point's gradient was off by
    100 % until such nodes were recomputed in FP64; per point and parameter
    (natural scale s, q, rho, 1, rho, rho, relative to mu) the mixed gradient
    must stay within 1e-4 of FP64."""
    import bench
    off, t, cv = bench.draw_batched(256, 3, 1000, 1000, 64)
    cot = np.random.default_rng(3).normal(size=len(t))
    g64, _ = C.mag_lc_batched_vjp(off, t, cv, cot, precision="fp64", **LC)
    g32, _ = C.mag_lc_batched_vjp(off, t, cv, cot, precision="mixed", **LC)
    g64, g32 = g64.cpu().numpy(), g32.cpu().numpy()
    reln = np.linalg.norm(g32 - g64, axis=1) / np.linalg.norm(g64, axis=1)
    assert reln.max() < 1e-4, (int(reln.argmax()), reln.max())
    c = 7
    tt, p = t[off[c]:off[c + 1]], cv[c]
    w = bench.trajectory(tt, p)
    per = {}
    for prec in ("fp64", "mixed"):
        m, g = C.mag_extended_source_grad(w, p[2], nlenses=2, s=p[0], q=p[1], u1=p[3], precision=prec, **LC)
        per[prec] = (np.asarray(m), np.asarray(g))  # NumPy in, NumPy out
    nat = np.array([p[0], p[1], p[2], 1.0, p[2], p[2]])
    err = np.abs(per["mixed"][1] - per["fp64"][1]) * nat / per["fp64"][0][:, None]
    assert err.max() < 1e-4, (np.unravel_index(err.argmax(), err.shape), err.max())


def _ambiguous(z, w, lens):
    res = np.abs(O.lens_eq(z, lens) - w[None, :])
    return np.any((res > 1e-6 / 30) & (res < 1e-6 * 30), axis=0)


def triple_workload(nsys=1000, npts=1000, seed=1):
    """The triple point-source workload: per system s1, s2 ~ U[0.5, 2], q1 ~
    logU[1e-4, 1], q2 ~ logU[1e-4, 1e-1], psi ~ U[0, 2 pi], then positions x and
    y ~ U[-1.5, 1.5] (the draw of tests/golden/make_golden.py)."""
    rng = np.random.default_rng(seed)
    s1 = rng.uniform(0.5, 2.0, nsys)
    s2 = rng.uniform(0.5, 2.0, nsys)
    q1 = 10 ** rng.uniform(-4, 0, nsys)
    q2 = 10 ** rng.uniform(-4, -1, nsys)
    psi = rng.uniform(0, 2 * np.pi, nsys)
    x = rng.uniform(-1.5, 1.5, (nsys, npts))
    y = rng.uniform(-1.5, 1.5, (nsys, npts))
    return s1, s2, q1, q2, psi, x + 1j * y


def root_bound(c, z, floor=1e-10):
    """Per-root tolerance on the relative root distance: 1e-10, or 64 eps times
    the root's relative condition number sum|a_k||z|^k / (|z| |p'(z)|) where
    that is larger (near-multiple roots, as around a lens of tiny mass, are
    determined by FP64 coefficients only to ~sqrt(eps))."""
    c = np.asarray(c)  # [n, deg+1] low -> high
    z = np.asarray(z)  # [n, deg]
    k = np.arange(c.shape[1])
    zp = z[..., None] ** k  # [n, deg, deg+1]
    b = (np.abs(c)[:, None, :] * np.abs(zp)).sum(-1)
    dp = (c[:, None, 1:] * k[1:] * zp[..., :-1]).sum(-1)
    kappa = b / np.maximum(np.abs(z) * np.abs(dp), 1e-300)
    return np.maximum(floor, 64 * 2.220446049250313e-16 * kappa)


def test_triple_point_source_1000_systems(G):
    d = G("mag_ps_triple_1000sys")
    s1, s2, q1, q2, psi, w = triple_workload()
    npos, nroots = int(d["npos"]), d["roots"].shape[1]
    errs = []
    for k in range(1000):
        p = dict(s=s1[k], q=q1[k], q3=q2[k], r3=s2[k], psi=psi[k])
        m, z, mask = C.mag_point_source(w[k, :npos], nlenses=3, precision="fp64", return_images=True, **p)
        lens = O.Lens.triple(p["s"], p["q"], p["q3"], p["r3"], p["psi"])
        wk = w[k, :npos] + lens.x_cm
        amb = _ambiguous(np.moveaxis(z, -1, 0), wk, lens) | d["ambiguous"][k]
        cnt = np.array([bin(int(x)).count("1") for x in mask])
        assert np.array_equal(cnt[~amb], d["nimg"][k][~amb]), k
        errs.append(rel(m[~amb], d["mag"][k][~amb]))
        # roots as sets against the reference solver's
        zr = d["roots"][k]
        dist = np.min(np.abs(zr[:, :, None] - z[:nroots, None, :]), axis=-1) / np.maximum(np.abs(zr), 1.0)
        c = C.lens_polynomial(w[k, :nroots], nlenses=3, **p)
        assert np.all(dist <= root_bound(c, zr)), k
    errs = np.concatenate(errs)
    # the promised bound everywhere; images next to a lens of mass fraction
    # ~1e-4, and near-caustic points (1/det J), amplify coefficient rounding
    assert errs.max() < 1e-4
    assert np.median(errs) < 1e-12 and np.quantile(errs, 0.9) < 1e-9


def test_lens_polynomial_matches_reference_coefficients(G):
    d = G("coeffs_triple")
    for k in range(len(d["s1"])):
        p = dict(s=d["s1"][k], q=d["q1"][k], q3=d["q2"][k], r3=d["s2"][k], psi=d["psi"][k])
        xcm = 0.5 * p["s"] * (1 - p["q"]) / (1 + p["q"])
        c = C.lens_polynomial(d["w"][k] - xcm, nlenses=3, **p)  # the fixture's positions are shifted already
        ref = d["coeffs"][k][:, ::-1]
        assert np.max(np.abs(c - ref)) <= 1e-12 * np.max(np.abs(ref))


def _min_mass_fraction(q1, q2):
    e1 = q1 / (1 + q1 + q2)
    return np.minimum(np.minimum(e1, q1 * e1), 1 - e1 - q1 * e1)


def test_triple_mixed_precision_routes_small_masses_to_fp64():
    """Where a mass fraction is below 1e-2, FP32 cannot separate the images
    clustered around that lens; the magnification kernels then run the FP64
    solver under "mixed" and return the FP64 result exactly."""
    s1, s2, q1, q2, psi, w = triple_workload()
    for k in np.flatnonzero(_min_mass_fraction(q1, q2) < 1e-2)[:50]:
        p = dict(s=s1[k], q=q1[k], q3=q2[k], r3=s2[k], psi=psi[k])
        m32 = C.mag_point_source(w[k], nlenses=3, precision="mixed", **p)
        m64 = C.mag_point_source(w[k], nlenses=3, precision="fp64", **p)
        assert np.array_equal(m32, m64, equal_nan=True), k


def test_triple_mixed_solver_against_fp64_full_workload():
    """Every position of the triple workload's systems whose mass fractions
    all reach 1e-2 (those that keep the mixed solver; the others go to FP64,
    above): the mixed solver (FP32 Aberth, compensated double-float stage,
    FP64 Newton polish) against the FP64 solver on the same polynomials
    (coefficients from cgb_lens_polynomial): roots as sets (relative distance
    within root_bound), image counts equal outside the ambiguous band,
    magnifications within the promised 1e-4."""
    s1, s2, q1, q2, psi, w = triple_workload()
    dev = torch.device("cuda", 0)
    worst_mu, mismatch = 0.0, 0
    for k in np.flatnonzero(_min_mass_fraction(q1, q2) >= 1e-2):
        p = dict(s=s1[k], q=q1[k], q3=q2[k], r3=s2[k], psi=psi[k])
        c = C.lens_polynomial(torch.as_tensor(w[k], device=dev), nlenses=3, **p)
        z64 = C.ehrlich_aberth(c, None, itmax=2500, precision="fp64").reshape(-1, 10).cpu().numpy()
        z32 = C.ehrlich_aberth(c, None, itmax=2500, precision="mixed").reshape(-1, 10).cpu().numpy()
        dist = np.min(np.abs(z64[:, :, None] - z32[:, None, :]), axis=-1) / np.maximum(np.abs(z64), 1.0)
        assert np.all(dist <= root_bound(c.cpu().numpy(), z64)), k
        lens = O.Lens.triple(p["s"], p["q"], p["q3"], p["r3"], p["psi"])
        wc = w[k] + lens.x_cm
        res64 = np.abs(O.lens_eq(z64.T, lens) - wc[None, :])
        res32 = np.abs(O.lens_eq(z32.T, lens) - wc[None, :])
        # a residual of either solver within x30 of the 1e-6 filter (CGB_ST_AMBIGUOUS)
        amb = np.any((res64 > 1e-6 / 30) & (res64 < 1e-6 * 30), axis=0) | \
            np.any((res32 > 1e-6 / 30) & (res32 < 1e-6 * 30), axis=0)
        n64, n32 = (res64 < 1e-6).sum(0), (res32 < 1e-6).sum(0)
        mismatch += int((n64[~amb] != n32[~amb]).sum())
        mu = lambda z, res: np.where(res < 1e-6, 1.0 / np.abs(O.lens_eq_det_jac(z, lens)), 0.0).sum(0)
        worst_mu = max(worst_mu, float(rel(mu(z32.T, res32)[~amb], mu(z64.T, res64)[~amb]).max()))
    assert mismatch == 0
    assert worst_mu < 1e-4


@pytest.mark.parametrize("n", range(4))
def test_triple_hexadecapole_routing(G, n):
    """Triple-lens routing in mag() (triple_routing="reference") against the
    reference's own triple hexadecapole and triple proximity test: route exact,
    hexadecapole magnification 1e-8 where it is accepted; the default
    integrates every point and agrees with the reference's
    mag_extended_source; with the third lens where the lens equation puts it
    ("corrected") the test rejects the accepted points where the hexadecapole
    is off by more than 10 % (all but at most one)."""
    d = G(f"hex_triple{n}")
    p = dict(s=float(d["s"]), q=float(d["q"]), q3=float(d["q3"]), r3=float(d["r3"]), psi=float(d["psi"]))
    rho = float(d["rho"])
    lens = O.Lens.triple(p["s"], p["q"], p["q3"], p["r3"], p["psi"])
    amb = _ambiguous(d["z"], d["w"] + lens.x_cm, lens)
    m, route = C.mag(d["w"], rho, nlenses=3, npts_limb=200, triple_routing="reference", return_route=True, **p)
    assert np.array_equal(route[~amb], ~d["test_prox"][~amb])
    ok = d["test_prox"] & ~amb & ~route
    assert ok.sum() > 10
    assert rel(m[ok], d["mu_multi"][ok]).max() < 1e-8  # images next to a mass fraction ~1e-4 amplify rounding
    m0, route0 = C.mag(d["w"], rho, nlenses=3, npts_limb=200, return_route=True, **p)
    assert route0.all()
    acc = d["full_idx"]
    assert rel(m0[acc], d["mag_full"]).max() < 1e-4
    _, routec = C.mag(d["w"], rho, nlenses=3, npts_limb=200, triple_routing="corrected", return_route=True, **p)
    bad = acc[rel(d["mu_multi"][acc], d["mag_full"]) > 0.1]
    assert routec[bad].sum() >= len(bad) - 1
