"""Generate the golden fixtures in tests/golden/*.npz from the reference itself.

Test infrastructure.  Runs the reference's UNMODIFIED Python source
(``src/caustics`` of fbartolic/caustics) on the NumPy stand-in for JAX in
``tests/golden/jaxshim``, with ``caustics.ehrlich_aberth_primitive.poly_roots``
bound to the reference's own compiled C++ solver (``oracle/_ref/libref_ea.so``,
built by ``make -C oracle ref`` from lib/ehrlich_aberth/ehrlich_aberth.h).

Only the container that holds the reference checkout can run this script; the
fixtures it writes are committed and are all that the tests read.

Known deviations of this harness from the reference under real JAX:
* the warm-start jitter of the refinement solves (extended_source.py:79-98) is
  a documented fixed +-0.5e-6 pattern (tests/golden/jaxshim/jax/random.py), not
  JAX's threefry stream, which cannot be reproduced here; the oracle and the
  kernels use the same pattern;
* roots come from the reference's C++ solver through ctypes instead of an XLA
  custom call (identical code, compiled with g++ -O2 -DNDEBUG).

The reference checkout is --ref, else $CAUSTICS_REF, else a directory named
`reference` beside this repository.

Usage:  python tests/golden/make_golden.py [--ref CHECKOUT] [--only NAME] [--procs N]
        (NAME: one fixture group, e.g. roots_jvp, likelihood, parallax, lc_2000pt,
        batched_seed2, batched_seed2_flagged, vjp_seed3, triple_ps_1000sys, hex_triple)
"""
import argparse
import ctypes
import os
import subprocess
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def default_reference():
    for cand in (os.environ.get("CAUSTICS_REF"), os.path.join(os.path.dirname(REPO), "reference")):
        if cand and os.path.isdir(os.path.join(cand, "src", "caustics")):
            return cand
    return None


def load_reference(ref_root):
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", f"REF={ref_root}"])
    lib = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libref_ea.so"))
    lib.ref_ea_solve.restype = ctypes.c_int
    lib.ref_ea_solve.argtypes = [ctypes.c_int] * 5 + [ctypes.c_void_p] * 3

    sys.path.insert(0, os.path.join(HERE, "jaxshim"))
    import jax.numpy as jnp  # the stand-in

    def poly_roots(coeffs, itmax=2000, compensated=False, custom_init=False, roots_init=None):
        # same contract as src/caustics/ehrlich_aberth_primitive.py:34-94
        coeffs = np.asarray(coeffs, dtype=np.complex128)
        ncoeffs = coeffs.shape[-1]
        out_shape = coeffs.shape[:-1] + (ncoeffs - 1,)
        flat = np.ascontiguousarray(coeffs.reshape(-1, ncoeffs)[:, ::-1])
        size = flat.shape[0]
        if custom_init:
            init = np.ascontiguousarray(np.asarray(roots_init, dtype=np.complex128).reshape(size, ncoeffs - 1))
        else:
            init = np.zeros((size, ncoeffs - 1), dtype=np.complex128)
        roots = np.zeros((size, ncoeffs - 1), dtype=np.complex128)
        rc = lib.ref_ea_solve(size, ncoeffs - 1, int(itmax), int(bool(compensated)), int(bool(custom_init)),
                              flat.ctypes.data, init.ctypes.data, roots.ctypes.data)
        assert rc == 0
        return jnp.asarray(roots.reshape(out_shape))

    mod = types.ModuleType("caustics.ehrlich_aberth_primitive")
    mod.poly_roots = poly_roots
    sys.modules["caustics.ehrlich_aberth_primitive"] = mod
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import caustics  # noqa: F401
    return lib, poly_roots


def binary_ps_points(n=10000):
    # binary point-source workload (s = 0.9, q = 0.1): x then y, each U[-1.5, 1.5], seed 0
    rng = np.random.default_rng(0)
    x = rng.uniform(-1.5, 1.5, n)
    y = rng.uniform(-1.5, 1.5, n)
    return x + 1j * y


def triple_ps_systems(nsys, npts, seed=1):
    # triple point-source workload: per-system s1,s2~U[.5,2], q1~logU[1e-4,1],
    # q2~logU[1e-4,1e-1], psi~U[0,2pi]; positions U[-1.5,1.5]^2 (x then y)
    rng = np.random.default_rng(seed)
    s1 = rng.uniform(0.5, 2.0, nsys)
    s2 = rng.uniform(0.5, 2.0, nsys)
    q1 = 10 ** rng.uniform(-4, 0, nsys)
    q2 = 10 ** rng.uniform(-4, -1, nsys)
    psi = rng.uniform(0, 2 * np.pi, nsys)
    x = rng.uniform(-1.5, 1.5, (nsys, npts))
    y = rng.uniform(-1.5, 1.5, (nsys, npts))
    return s1, s2, q1, q2, psi, x + 1j * y


def near_caustic_points(caustic, rho, n, seed):
    rng = np.random.default_rng(seed)
    c = np.asarray(caustic).reshape(-1)
    idx = rng.choice(len(c), size=n, replace=False)
    phi = rng.uniform(-np.pi, np.pi, n)
    r = rng.uniform(0.0, 2 * rho, n)
    return c[idx] + r * np.exp(1j * phi)


def roots_jvp_fixture(poly_roots, ps):
    """Derivatives of the reference solver's roots along random coefficient
    tangents, by central differences of the reference solver itself (step 1e-7
    relative, roots matched to the unperturbed ones): the known answer for the
    primitive's implicit-function JVP (ehrlich_aberth_primitive.py:252-312),
    whose JAX evaluation is not available."""
    rng = np.random.default_rng(21)
    w = rng.uniform(-1.2, 1.2, 24) + 1j * rng.uniform(-1.2, 1.2, 24)
    out = {}
    polys = {"5": np.asarray(ps._poly_coeffs_binary(w, 0.45, 1 / 1.1))}
    # a triple system without a tiny-mass lens (clustered roots are outside the
    # linear regime of any finite difference): s=1, q=0.5, q3=0.3, r3=0.9, psi=1.1
    e1 = 0.5 / 1.8
    polys["10"] = np.asarray(ps._poly_coeffs_triple(w, 0.5, 0.9 * np.exp(1.1j), e1, 0.5 * e1))
    for deg, c in polys.items():
        lo = c[:, ::-1].copy()  # low -> high, as the primitive takes them
        dp = (rng.normal(size=lo.shape) + 1j * rng.normal(size=lo.shape)) * np.abs(lo)
        z = np.asarray(poly_roots(c, itmax=2500)).reshape(len(c), -1)
        h = 1e-7
        zp = np.asarray(poly_roots((lo + h * dp)[:, ::-1], itmax=2500)).reshape(len(c), -1)
        zm = np.asarray(poly_roots((lo - h * dp)[:, ::-1], itmax=2500)).reshape(len(c), -1)
        match = lambda zz: np.take_along_axis(zz, np.argmin(np.abs(zz[:, None, :] - z[:, :, None]), axis=2), axis=1)
        out["p" + deg], out["dp" + deg], out["z" + deg] = lo, dp, z
        out["dz" + deg] = (match(zp) - match(zm)) / (2 * h)
    return out


def likelihood_fixture():
    """marginalized_log_likelihood (linalg.py:10-94, diagonal covariance) on
    three light curves of uneven length: the list total and each curve alone."""
    from caustics import linalg as la
    rng = np.random.default_rng(31)
    lens = [150, 400, 37]
    A, f, c = [], [], []
    for n, (fs, fb, sig) in zip(lens, [(2.0, 0.5, 0.05), (0.7, 1.3, 0.02), (5.0, -0.2, 0.3)]):
        a = 1.0 + 3.0 * np.abs(rng.normal(size=n))
        A.append(a)
        f.append(fs * a + fb + sig * rng.normal(size=n))
        c.append(np.full(n, 1.0 / sig ** 2) * rng.uniform(0.5, 1.5, n))
    beta, ll = la.marginalized_log_likelihood(A, f, c)
    ll_each = np.array([float(la.marginalized_log_likelihood([a], [ff], [cc])[1]) for a, ff, cc in zip(A, f, c)])
    return dict(offsets=np.concatenate([[0], np.cumsum(lens)]).astype(np.int64), A=np.concatenate(A),
                fobs=np.concatenate(f), C_inv=np.concatenate(c), beta=np.stack([np.asarray(b) for b in beta]),
                ll=np.float64(ll), ll_each=ll_each)


def parallax_fixture():
    """AnnualParallaxTrajectory.compute (trajectory.py:106-157) with a synthetic
    projected Sun ephemeris (astropy, which the constructor needs, is absent:
    its module is stubbed for the import and the ephemeris attributes are set
    directly, as _compute_sun_position_and_velocity would)."""
    for name in ("astropy", "astropy.coordinates", "astropy.time"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["astropy.coordinates"].get_body_barycentric_posvel = None
    sys.modules["astropy.time"].Time = None
    from caustics import trajectory as tr
    t_jpl = np.arange(8000.0, 8400.0 + 1, 1.0)
    ph = 2 * np.pi * (t_jpl - 8123.4) / 365.25
    s_e, s_n = 0.98 * np.cos(ph), 0.41 * np.sin(ph) + 0.05
    s_e_dot, s_n_dot = -0.98 * np.sin(ph) * 2 * np.pi / 365.25, 0.41 * np.cos(ph) * 2 * np.pi / 365.25
    traj = object.__new__(tr.AnnualParallaxTrajectory)
    traj.t_jpl, traj.s_e, traj.s_n, traj.s_e_dot, traj.s_n_dot = t_jpl, s_e, s_n, s_e_dot, s_n_dot
    t = np.sort(np.random.default_rng(41).uniform(8001.0, 8399.0, 300))
    out = dict(t_jpl=t_jpl, s_e=s_e, s_n=s_n, s_e_dot=s_e_dot, s_n_dot=s_n_dot, t=t)
    cases = [dict(u0=0.1, t0=8200.3, tE=35.0, piEE=0.2, piEN=-0.15), dict(u0=-0.05, t0=8150.0, tE=80.0, piEE=-0.4, piEN=0.3)]
    for k, c in enumerate(cases):
        w = np.asarray(traj.compute(t, **dict(c)))
        out[f"w{k}"] = w
        out[f"params{k}"] = np.array([c["u0"], c["t0"], c["tE"], c["piEE"], c["piEN"]])
    return out


# ---------------------------------------------------------------------------
# Fixtures at the configured workload sizes.  The reference evaluates one
# extended-source point in ~0.2-0.35 s on the stand-in, so these spread the
# points over a spawn pool whose workers each load the reference.
# ---------------------------------------------------------------------------

def _worker_init(ref_root):
    load_reference(ref_root)


def pool_map(fn, jobs, ref_root, procs):
    import multiprocessing as mp
    if procs <= 1:
        _worker_init(ref_root)
        return [fn(j) for j in jobs]
    with mp.get_context("spawn").Pool(procs, initializer=_worker_init, initargs=(ref_root,)) as pool:
        return pool.map(fn, jobs, chunksize=1)


def _job_lc_mag(job):
    """The reference's mag() (lightcurve.py:99-254) on a chunk of source positions."""
    w, rho, kw = job
    from caustics import lightcurve as lc
    return np.asarray(lc.mag(np.asarray(w), rho, nlenses=2, **kw), dtype=np.float64)


def _job_triple_ps(job):
    """mag_point_source and the image solve of one triple system (point_source.py:1652-1830)."""
    w, s, q, q3, r3, psi = job
    from caustics import point_source as ps
    a, e1 = 0.5 * s, q / (1 + q + q3)
    e2, r3c, xcm = q * e1, r3 * np.exp(1j * psi), 0.5 * s * (1 - q) / (1 + q)
    mag = np.asarray(ps.mag_point_source(w.copy(), nlenses=3, s=s, q=q, q3=q3, r3=r3, psi=psi))
    z, m = ps._images_point_source(w + xcm, nlenses=3, a=a, r3=r3c, e1=e1, e2=e2)
    return mag, np.asarray(z), np.asarray(m)


def _job_es_triple(job):
    w0, rho, kw = job
    from caustics import extended_source as es
    return float(es.mag_extended_source(w0, rho, nlenses=3, **kw))


def lc_mag_pooled(w, rho, kw, ref_root, procs, chunk=25):
    w = np.asarray(w)
    jobs = [(w[i:i + chunk], rho, kw) for i in range(0, len(w), chunk)]
    return np.concatenate(pool_map(_job_lc_mag, jobs, ref_root, procs)) if len(w) else np.zeros(0)


def reference_route(w, rho, s, q):
    """The reference's routing in mag() (lightcurve.py:200-224), from its own
    pieces: True where the point takes the contour integral."""
    from caustics import lightcurve as lc
    from caustics import multipole as mp
    from caustics import point_source as ps
    a, e1 = 0.5 * s, 1 / (1 + q)
    xcm = a * (1 - q) / (1 + q)
    wc = np.asarray(w) + xcm
    z, m = ps._images_point_source(wc, nlenses=2, roots_itmax=2500, a=a, e1=e1)
    _, dmu = mp._mag_hexadecapole(z, m, rho, nlenses=2, a=a, e1=e1)
    t1 = np.asarray(lc._caustics_proximity_test(wc, z, m, rho, dmu, nlenses=2, a=a, e1=e1))
    t2 = np.asarray(lc._planetary_caustic_test(wc, rho, a=a, e1=e1))
    return ~((t1 & t2) if q < 0.01 else t1)


def trajectory_points(t, cv):
    """w(t) of one curve (s, q, rho, u1, u0, alpha, t0, tE): the rectilinear
    part of trajectory.py:152-155 (pi_E = 0)."""
    u0, al, t0, te = cv[4], cv[5], cv[6], cv[7]
    tau = (np.asarray(t) - t0) / te
    return (u0 * np.cos(al) + tau * np.sin(al)) + 1j * (-u0 * np.sin(al) + tau * np.cos(al))


def batched_workload(seed, ncurves, nmin, nmax):
    sys.path.insert(0, REPO)
    from bench import draw_batched
    return draw_batched(ncurves, seed, nmin, nmax, ncurves)


def lc_2000pt_fixture(ref, procs):
    """Every point of the 2000-point limb-darkened light curve (s 1.1, q 5e-3,
    rho 1e-2, u1 0.5, npts_limb 500, npts_ld 100, u0 0.05, alpha 0.6, t0 0,
    tE 20, t uniform on [-40, 40])."""
    t = np.linspace(-40.0, 40.0, 2000)
    cv = np.array([1.1, 5e-3, 1e-2, 0.5, 0.05, 0.6, 0.0, 20.0])
    w = trajectory_points(t, cv)
    kw = dict(npts_limb=500, limb_darkening=True, u1=0.5, npts_ld=100, s=1.1, q=5e-3)
    mag = lc_mag_pooled(w, 1e-2, kw, ref, procs)
    return {"mag_lc_binary_ld_s1.1_q5e-3_2000pt": dict(t=t, w=w, curve=cv, npts_limb=np.int64(500),
                                                       npts_ld=np.int64(100), mag=mag,
                                                       route=reference_route(w, 1e-2, 1.1, 5e-3))}


def _batched_points_fixture(off, t, cv, curve_ids, ref, procs):
    """mag() of the given curves of a batched workload, npts_limb 200, npts_ld
    100, limb darkened with each curve's u1."""
    ts, mags, routes, lens = [], [], [], []
    for c in curve_ids:
        tc = t[off[c]:off[c + 1]]
        w = trajectory_points(tc, cv[c])
        kw = dict(npts_limb=200, limb_darkening=True, u1=float(cv[c, 3]), npts_ld=100, s=float(cv[c, 0]),
                  q=float(cv[c, 1]))
        mags.append(lc_mag_pooled(w, float(cv[c, 2]), kw, ref, procs))
        routes.append(reference_route(w, float(cv[c, 2]), float(cv[c, 0]), float(cv[c, 1])))
        ts.append(tc)
        lens.append(len(tc))
        print(f"[golden] curve {c}: {len(tc)} points, {int(routes[-1].sum())} contour", flush=True)
    return dict(curve_ids=np.asarray(curve_ids, dtype=np.int64), offsets=np.concatenate([[0], np.cumsum(lens)]).astype(
        np.int64), t=np.concatenate(ts), curves=cv[np.asarray(curve_ids)], mag=np.concatenate(mags),
        route=np.concatenate(routes), npts_limb=np.int64(200), npts_ld=np.int64(100))


def batched_seed2_fixture(ref, procs):
    """Whole curves of the 4096-curve workload (seed 2, lengths U{200..5000}):
    the two shortest with q < 1e-3, with 1e-3 <= q < 1e-2 and with q >= 1e-2,
    and the shortest curve of at least 2000 points with q >= 1e-2."""
    off, t, cv = batched_workload(2, 4096, 200, 5000)
    lens, q = np.diff(off), cv[:, 1]
    pick = []
    for lo, hi in [(0.0, 1e-3), (1e-3, 1e-2), (1e-2, 2.0)]:
        idx = np.flatnonzero((q >= lo) & (q < hi))
        pick += [int(c) for c in idx[np.argsort(lens[idx], kind="stable")][:2]]
    idx = np.flatnonzero((q >= 1e-2) & (lens >= 2000))
    pick.append(int(idx[np.argmin(lens[idx])]))
    return {"mag_lc_batched_seed2_sample": _batched_points_fixture(off, t, cv, pick, ref, procs)}


def batched_seed2_flagged_fixture(ref, procs, flagged):
    """Single points of the 4096-curve workload (seed 2) given by their point
    index: the points whose evaluation set a non-convergence or contour-linking
    status bit in a full run of the GPU path."""
    off, t, cv = batched_workload(2, 4096, 200, 5000)
    pts = np.unique(np.asarray(flagged, dtype=np.int64))
    cid = np.searchsorted(off, pts, side="right") - 1
    ws = np.array([trajectory_points(t[i:i + 1], cv[c])[0] for i, c in zip(pts, cid)])
    jobs = [(ws[k:k + 1], float(cv[c, 2]), dict(npts_limb=200, limb_darkening=True, u1=float(cv[c, 3]), npts_ld=100,
                                                s=float(cv[c, 0]), q=float(cv[c, 1])))
            for k, c in enumerate(cid)]
    mags = np.concatenate(pool_map(_job_lc_mag, jobs, ref, procs))
    route = np.array([reference_route(ws[k:k + 1], float(cv[c, 2]), float(cv[c, 0]), float(cv[c, 1]))[0]
                      for k, c in enumerate(cid)])
    return {"mag_lc_batched_seed2_flagged": dict(point_ids=pts, curve_ids=cid, t=t[pts], curves=cv[cid], mag=mags,
                                                 route=route, npts_limb=np.int64(200), npts_ld=np.int64(100))}


def vjp_seed3_fixture(ref, procs, curve_ids=(3, 8, 5, 9)):
    """Per-point derivatives of the reference's mag() with respect to
    (s, q, rho, u1, Re w, Im w) by central differences at two steps, on four
    whole curves (1000 points each) of the 256-curve gradient workload (seed 3):
    curves 3 and 8 (q >= 0.01) and 5 and 9 (q < 0.01, every point through the
    contour integral).  Steps: h * |parameter| for s, q, rho, u1 and h * rho for
    the source position, h = 1e-7 and 1e-8; a derivative is trusted where the
    two steps agree (the discrete limb refinement can change between +-h)."""
    off, t, cv = batched_workload(3, 256, 1000, 1000)
    steps = (1e-7, 1e-8)
    out = {"curve_ids": np.asarray(curve_ids, dtype=np.int64), "steps": np.asarray(steps)}
    jobs, keys = [], []
    chunk = 50
    for c in curve_ids:
        w = trajectory_points(t[off[c]:off[c + 1]], cv[c])
        base = dict(npts_limb=200, limb_darkening=True, u1=float(cv[c, 3]), npts_ld=100, s=float(cv[c, 0]),
                    q=float(cv[c, 1]))
        rho = float(cv[c, 2])
        variants = [("base", 0, 0.0, 0)]
        for x in range(6):
            for h in steps:
                for sg in (1, -1):
                    variants.append(("d", x, h, sg))
        for v in variants:
            _, x, h, sg = v
            kw, r, ww = dict(base), rho, w
            if v[0] == "d":
                if x == 0:
                    kw["s"] = base["s"] * (1 + sg * h)
                elif x == 1:
                    kw["q"] = base["q"] * (1 + sg * h)
                elif x == 2:
                    r = rho * (1 + sg * h)
                elif x == 3:
                    kw["u1"] = base["u1"] * (1 + sg * h)
                else:
                    ww = w + sg * h * rho * (1.0 if x == 4 else 1j)
            for i in range(0, len(w), chunk):
                jobs.append((ww[i:i + chunk], r, kw))
                keys.append((c, v, i))
    res = pool_map(_job_lc_mag, jobs, ref, procs)
    got = {}
    for k, m in zip(keys, res):
        got.setdefault((k[0], k[1]), []).append((k[2], m))
    for c in curve_ids:
        cat = lambda v: np.concatenate([m for _, m in sorted(got[(c, v)], key=lambda e: e[0])])
        mag = cat(("base", 0, 0.0, 0))
        J = np.zeros((2, len(mag), 6))
        scale = [cv[c, 0], cv[c, 1], cv[c, 2], cv[c, 3], cv[c, 2], cv[c, 2]]
        for x in range(6):
            for hi, h in enumerate(steps):
                J[hi, :, x] = (cat(("d", x, h, 1)) - cat(("d", x, h, -1))) / (2 * h * scale[x])
        w = trajectory_points(t[off[c]:off[c + 1]], cv[c])
        out[f"t{c}"] = t[off[c]:off[c + 1]]
        out[f"curve{c}"] = cv[c]
        out[f"mag{c}"] = mag
        out[f"jac{c}"] = J
        out[f"route{c}"] = reference_route(w, float(cv[c, 2]), float(cv[c, 0]), float(cv[c, 1]))
    return {"vjp_seed3_fd": out}


def triple_ps_1000sys_fixture(ref, procs, npos=32, nroots=2):
    """Triple-lens point source over all 1000 systems of the triple workload
    (seed 1: s1, s2 ~ U[0.5, 2], q1 ~ logU[1e-4, 1], q2 ~ logU[1e-4, 1e-1],
    psi ~ U[0, 2 pi]; 1000 positions per system, x then y ~ U[-1.5, 1.5]; the
    reference keywords s = s1, q = q1, q3 = q2, r3 = s2): magnifications and
    image counts of the first `npos` positions of every system, and roots with
    their image mask for the first `nroots`."""
    s1, s2, q1, q2, psi, w = triple_ps_systems(1000, 1000, seed=1)
    jobs = [(w[k, :npos].copy(), s1[k], q1[k], q2[k], s2[k], psi[k]) for k in range(1000)]
    res = pool_map(_job_triple_ps, jobs, ref, procs)
    mag = np.stack([r[0] for r in res])
    nimg = np.stack([r[2].sum(axis=0) for r in res]).astype(np.uint8)
    roots = np.stack([r[1][:, :nroots].T for r in res])  # [sys, pos, 10]
    mask = np.stack([r[2][:, :nroots].T for r in res])
    # positions where one of the reference's own image residuals lies within x30
    # of the 1e-6 filter threshold (point_source.py:1707): their count is decided
    # by rounding
    from caustics import point_source as ps
    amb = []
    for k, r in enumerate(res):
        a, e1 = 0.5 * s1[k], q1[k] / (1 + q1[k] + q2[k])
        prm = dict(a=a, r3=s2[k] * np.exp(1j * psi[k]), e1=e1, e2=q1[k] * e1)
        wc = w[k, :npos] + a * (1 - q1[k]) / (1 + q1[k])
        resid = np.abs(np.asarray(ps.lens_eq(r[1], nlenses=3, **prm)) - wc[None, :])
        amb.append(np.any((resid > 1e-6 / 30) & (resid < 1e-6 * 30), axis=0))
    return {"mag_ps_triple_1000sys": dict(npos=np.int64(npos), mag=mag, nimg=nimg, roots=roots, mask=mask,
                                          ambiguous=np.stack(amb))}


def hex_triple_fixture(ref, procs):
    """The reference's triple-lens hexadecapole (multipole.py:208-244) and the
    triple branch of its proximity test (lightcurve.py:23-75, third lens term
    (z + r3) as written there) on points near the caustics and elsewhere.  The
    reference's mag() never calls them for triple lenses (lightcurve.py:226-227)
    and fails on an undefined name after them (:252), so they are run directly,
    on the same inputs mag() would give them.  mag_full: the reference's
    uniform-source mag_extended_source (npts_limb 200) at up to 12 points per
    system that the test accepts, to show the hexadecapole's accuracy there."""
    from caustics import lightcurve as lc
    from caustics import multipole as mp
    from caustics import point_source as ps
    s1, s2, q1, q2, psi, _ = triple_ps_systems(1000, 1, seed=1)
    e1 = q1 / (1 + q1 + q2)
    e3 = 1 - e1 - q1 * e1
    systems = [(1.0, 0.5, 0.05, 0.9, 1.1, 1e-2)]
    good = np.flatnonzero((np.minimum(np.minimum(e1, q1 * e1), e3) >= 1e-2))[:2]
    small = np.flatnonzero(np.minimum(np.minimum(e1, q1 * e1), e3) < 1e-2)[:1]
    for k, rho in zip(list(good) + list(small), (1e-2, 3e-3, 3e-3)):
        systems.append((s1[k], q1[k], q2[k], s2[k], psi[k], rho))
    out = {}
    for n, (s, q, q3, r3, ps_, rho) in enumerate(systems):
        a, ee1 = 0.5 * s, q / (1 + q + q3)
        ee2, r3c, xcm = q * ee1, r3 * np.exp(1j * ps_), 0.5 * s * (1 - q) / (1 + q)
        _, cau = ps.critical_and_caustic_curves(npts=100, nlenses=3, s=s, q=q, q3=q3, r3=r3, psi=ps_)
        rng = np.random.default_rng(50 + n)
        wpts = np.concatenate([near_caustic_points(cau, 10 * rho, 60, seed=60 + n),
                               rng.uniform(-1, 1, 20) + 1j * rng.uniform(-1, 1, 20)])
        prm = dict(a=a, r3=r3c, e1=ee1, e2=ee2)
        z, m = ps._images_point_source(wpts + xcm, nlenses=3, **prm)
        mu, dmu = mp._mag_hexadecapole(z, m, rho, nlenses=3, **prm)
        t1 = np.asarray(lc._caustics_proximity_test(wpts + xcm, z, m, rho, dmu, nlenses=3, **prm))
        acc = np.flatnonzero(t1)[:12]
        mfull = pool_map(_job_es_triple, [(wpts[i], rho, dict(npts_limb=200, s=s, q=q, q3=q3, r3=r3, psi=ps_))
                                          for i in acc], ref, procs)
        out[f"hex_triple{n}"] = dict(s=np.float64(s), q=np.float64(q), q3=np.float64(q3), r3=np.float64(r3),
                                     psi=np.float64(ps_), rho=np.float64(rho), w=wpts, z=np.asarray(z),
                                     mask=np.asarray(m), mu_multi=np.asarray(mu), delta_mu=np.asarray(dmu),
                                     test_prox=t1, full_idx=acc, mag_full=np.asarray(mfull))
        print(f"[golden] triple hexadecapole system {n}: {int(t1.sum())} of {len(t1)} accepted", flush=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=default_reference())
    ap.add_argument("--only", default=None, help="write only this fixture group (see the module docstring)")
    ap.add_argument("--procs", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--flagged", default=None, help="batched_seed2_flagged: .npy of point indices")
    args = ap.parse_args()
    if args.ref is None:
        raise SystemExit("no reference checkout: pass --ref or set CAUSTICS_REF")
    big = {"lc_2000pt": lambda: lc_2000pt_fixture(args.ref, args.procs),
           "batched_seed2": lambda: batched_seed2_fixture(args.ref, args.procs),
           "batched_seed2_flagged": lambda: batched_seed2_flagged_fixture(args.ref, args.procs, np.load(args.flagged)),
           "vjp_seed3": lambda: vjp_seed3_fixture(args.ref, args.procs),
           "triple_ps_1000sys": lambda: triple_ps_1000sys_fixture(args.ref, args.procs),
           "hex_triple": lambda: hex_triple_fixture(args.ref, args.procs)}
    lib, poly_roots = load_reference(args.ref)
    if args.only in big:
        t0 = time.time()
        for name, d in big[args.only]().items():
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
            print(f"[golden] wrote {name} in {time.time() - t0:.1f}s", flush=True)
        return
    from caustics import point_source as ps
    if args.only == "roots_jvp":
        np.savez_compressed(os.path.join(HERE, "roots_jvp.npz"), **roots_jvp_fixture(poly_roots, ps))
        return
    if args.only == "parallax":
        np.savez_compressed(os.path.join(HERE, "parallax.npz"), **parallax_fixture())
        return
    if args.only == "likelihood":
        np.savez_compressed(os.path.join(HERE, "likelihood.npz"), **likelihood_fixture())
        return
    from caustics import extended_source as es
    from caustics import lightcurve as lc
    from caustics import multipole as mp
    from caustics import utils as ut
    out = {}
    t0 = time.time()

    # ---- coefficients (point_source.py:17-86, 89-1479) ----
    rng = np.random.default_rng(11)
    w = rng.uniform(-1.5, 1.5, 64) + 1j * rng.uniform(-1.5, 1.5, 64)
    cb = np.stack([np.asarray(ps._poly_coeffs_binary(w, a, e1)) for a, e1 in [(0.45, 1 / 1.1), (0.55, 0.9), (1.2, 0.5)]])
    out["coeffs_binary"] = dict(w=w, a=np.array([0.45, 0.55, 1.2]), e1=np.array([1 / 1.1, 0.9, 0.5]), coeffs=cb)
    s1, s2, q1, q2, psi, wt = triple_ps_systems(6, 16, seed=1)
    ct = []
    for k in range(6):
        a, e1 = 0.5 * s1[k], q1[k] / (1 + q1[k] + q2[k])
        e2, r3 = q1[k] * e1, s2[k] * np.exp(1j * psi[k])
        ct.append(np.asarray(ps._poly_coeffs_triple(wt[k], a, r3, e1, e2)))
    out["coeffs_triple"] = dict(s1=s1, s2=s2, q1=q1, q2=q2, psi=psi, w=wt, coeffs=np.stack(ct))

    # ---- roots: binary point-source polynomials through the reference solver (ehrlich_aberth.h) ----
    wc = binary_ps_points()[:2000]
    a, q = 0.45, 0.1
    e1 = 1 / (1 + q)
    xcm = a * (1 - q) / (1 + q)
    coeffs = np.asarray(ps._poly_coeffs_binary(wc + xcm, a, e1))
    out["roots_binary_s0.9_q0.1"] = dict(w=wc, coeffs=coeffs,
                             roots_plain=np.asarray(poly_roots(coeffs, itmax=2500)),
                             roots_comp=np.asarray(poly_roots(coeffs, itmax=2500, compensated=True)))
    # the reference's own fixture (tests/test_ehrlich_aberth_primitive.py:19-27)
    wf = np.linspace(0.3, 0.35, 10).astype(np.complex128)
    cf = np.asarray(ps._poly_coeffs_binary(wf, 0.45, 0.8))
    out["roots_fixture"] = dict(w=wf, coeffs=cf, roots_plain=np.asarray(poly_roots(cf)),
                                roots_comp=np.asarray(poly_roots(cf, compensated=True)))

    # ---- point-source magnification (point_source.py:1762-1830) ----
    wfull = binary_ps_points()
    out["mag_ps_binary_s0.9_q0.1"] = dict(w=wfull, s=np.float64(0.9), q=np.float64(0.1),
                              mag=np.asarray(ps.mag_point_source(wfull.copy(), nlenses=2, s=0.9, q=0.1)))
    xg = np.linspace(-0.5, 0.5, 50)
    wg = (xg[None, :] + 1j * xg[:, None]).reshape(-1)
    out["mag_ps_grid"] = dict(w=wg, s=np.float64(0.9), q=np.float64(0.2),
                              mag=np.asarray(ps.mag_point_source(wg.copy(), nlenses=2, s=0.9, q=0.2)))
    s1, s2, q1, q2, psi, wt = triple_ps_systems(8, 64, seed=1)
    mt, zt, mk = [], [], []
    for k in range(8):
        mt.append(np.asarray(ps.mag_point_source(wt[k].copy(), nlenses=3, s=s1[k], q=q1[k], q3=q2[k], r3=s2[k], psi=psi[k])))
        a, e1 = 0.5 * s1[k], q1[k] / (1 + q1[k] + q2[k])
        z, m = ps._images_point_source(wt[k] + a * (1 - q1[k]) / (1 + q1[k]), nlenses=3, a=a,
                                       r3=s2[k] * np.exp(1j * psi[k]), e1=e1, e2=q1[k] * e1)
        zt.append(np.asarray(z)); mk.append(np.asarray(m))
    out["mag_ps_triple"] = dict(s1=s1, s2=s2, q1=q1, q2=q2, psi=psi, w=wt, mag=np.stack(mt),
                                z=np.stack(zt), mask=np.stack(mk))
    print(f"[golden] point source done {time.time() - t0:.1f}s", flush=True)

    # ---- critical curves and caustics (point_source.py:1582-1649) ----
    zcr, zca = ps.critical_and_caustic_curves(npts=50, nlenses=2, s=0.9, q=0.2)
    out["caustics_binary"] = dict(s=np.float64(0.9), q=np.float64(0.2), npts=np.int64(50),
                                  z_cr=np.asarray(zcr), z_ca=np.asarray(zca))

    # ---- hexadecapole + proximity tests (multipole.py, lightcurve.py:23-85) ----
    hx = {}
    for tag, (s, q, rho) in {"q0.2": (0.9, 0.2, 1e-2), "q5e-3": (1.1, 5e-3, 1e-2), "q0.05": (1.3, 0.05, 3e-3)}.items():
        a, e1 = 0.5 * s, 1 / (1 + q)
        xcm = a * (1 - q) / (1 + q)
        _, cau = ps.critical_and_caustic_curves(npts=60, nlenses=2, s=s, q=q)
        wpts = np.concatenate([near_caustic_points(cau, 10 * rho, 80, seed=5),
                               np.random.default_rng(6).uniform(-1, 1, 40) + 1j * np.random.default_rng(7).uniform(-1, 1, 40)])
        z, m = ps._images_point_source(wpts + xcm, nlenses=2, a=a, e1=e1)
        mu, dmu = mp._mag_hexadecapole(z, m, rho, nlenses=2, a=a, e1=e1)
        t1 = lc._caustics_proximity_test(wpts + xcm, z, m, rho, dmu, nlenses=2, a=a, e1=e1)
        t2 = lc._planetary_caustic_test(wpts + xcm, rho, a=a, e1=e1)
        hx[tag] = dict(s=np.float64(s), q=np.float64(q), rho=np.float64(rho), w=wpts, z=np.asarray(z),
                       mask=np.asarray(m), mu_multi=np.asarray(mu), delta_mu=np.asarray(dmu),
                       test_prox=np.asarray(t1), test_planet=np.asarray(t2))
    for tag, d in hx.items():
        out["hex_" + tag] = d
    print(f"[golden] hexadecapole done {time.time() - t0:.1f}s", flush=True)

    # ---- KAT-style helpers (utils.py, extended_source.py:156-216) ----
    z = np.array([0.0, 1.0, 1.01, 1.02, 1.03, 0.0, 4.0, 4.01, 0.0, 0.0, 6.0]).astype(np.complex128)
    par = np.array([-1., -1., -1., 1., 1., 1., 1., 1., 1., 1., 1.])
    msk = np.array([0., 1., 1., 1., 1., 0., 1., 1., 0., 0., 1.])
    out["split_segment"] = dict(z=z, parity=par, mask=msk,
                                parts=np.asarray(es._split_segment(np.stack([z, par, msk]), n_parts=5)))

    # ---- limb images (extended_source.py:56-153) ----
    limb = {}
    for k, (w0, rho, npts) in enumerate([(0.1 + 0.05j, 0.05, 100), (-0.3 + 0.02j, 1e-2, 200), (0.35 + 0.0j, 0.1, 60)]):
        a, e1 = 0.45, 1 / 1.2
        zl, ml, pl = es._images_of_source_limb(w0 + a * (1 - 0.2) / 1.2, rho, nlenses=2, npts=npts, a=a, e1=e1)
        limb[f"limb{k}"] = dict(w0=np.complex128(w0), rho=np.float64(rho), npts=np.int64(npts), s=np.float64(0.9),
                                q=np.float64(0.2), z=np.asarray(zl), mask=np.asarray(ml), parity=np.asarray(pl))
    out.update(limb)

    # ---- extended source magnification (extended_source.py:741-904) ----
    _, cau = ps.critical_and_caustic_curves(npts=50, nlenses=2, s=0.9, q=0.2)
    cases = []
    for rho, npts_limb, ld, u1, seed in [(1e-1, 200, False, 0.0, 21), (1e-2, 300, False, 0.0, 22), (1e-3, 200, False, 0.0, 23),
                                         (1e-1, 200, True, 0.7, 24), (1e-2, 300, True, 0.7, 25), (5e-2, 100, True, 0.3, 26)]:
        wpts = np.concatenate([near_caustic_points(cau, rho, 5, seed), [0.6 + 0.4j]])
        mags = np.array([float(es.mag_extended_source(wv, rho, nlenses=2, npts_limb=npts_limb, limb_darkening=ld,
                                                         u1=u1, npts_ld=100, s=0.9, q=0.2)) for wv in wpts])
        cases.append(dict(w=wpts, rho=np.float64(rho), npts_limb=np.int64(npts_limb), ld=np.bool_(ld), u1=np.float64(u1),
                          s=np.float64(0.9), q=np.float64(0.2), mag=mags))
        print(f"[golden] mag_es rho={rho} ld={ld} {time.time() - t0:.1f}s", flush=True)
    for k, c in enumerate(cases):
        out[f"mag_es{k}"] = c

    # ---- light curve (lightcurve.py:99-254): the 2000-point LD light curve (s 1.1, q 5e-3), every 100th point, and a q>0.01 curve ----
    t = np.linspace(-40.0, 40.0, 2000)
    tau = t / 20.0
    u0, alpha = 0.05, 0.6
    wtraj = (u0 * np.cos(alpha) + tau * np.sin(alpha)) + 1j * (-u0 * np.sin(alpha) + tau * np.cos(alpha))
    sub = wtraj[::100]
    mags = np.asarray(lc.mag(sub, 1e-2, nlenses=2, npts_limb=500, limb_darkening=True, u1=0.5, npts_ld=100, s=1.1, q=5e-3))
    out["mag_lc_binary_ld_s1.1_q5e-3"] = dict(w=sub, rho=np.float64(1e-2), u1=np.float64(0.5), s=np.float64(1.1), q=np.float64(5e-3),
                              npts_limb=np.int64(500), npts_ld=np.int64(100), mag=mags)
    print(f"[golden] mag LD light curve {time.time() - t0:.1f}s", flush=True)
    wq = np.linspace(-0.8, 0.8, 24) + 0.08j
    mags = np.asarray(lc.mag(wq, 2e-2, nlenses=2, npts_limb=200, limb_darkening=True, u1=0.4, npts_ld=60, s=0.95, q=0.3))
    out["mag_lc_q0.3"] = dict(w=wq, rho=np.float64(2e-2), u1=np.float64(0.4), s=np.float64(0.95), q=np.float64(0.3),
                              npts_limb=np.int64(200), npts_ld=np.int64(60), mag=mags)
    print(f"[golden] mag q0.3 {time.time() - t0:.1f}s", flush=True)

    # ---- triple extended source (nlenses=3) ----
    s, q, q3, r3, psi = 1.0, 0.5, 0.05, 0.9, 1.1
    wpts = np.array([0.02 + 0.03j, -0.15 + 0.1j, 0.4 - 0.25j])
    mags = np.array([float(es.mag_extended_source(wv, 2e-2, nlenses=3, npts_limb=200, s=s, q=q, q3=q3, r3=r3, psi=psi))
                     for wv in wpts])
    out["mag_es_triple"] = dict(w=wpts, rho=np.float64(2e-2), npts_limb=np.int64(200), s=np.float64(s), q=np.float64(q),
                                q3=np.float64(q3), r3=np.float64(r3), psi=np.float64(psi), mag=mags)
    print(f"[golden] triple {time.time() - t0:.1f}s", flush=True)

    out["roots_jvp"] = roots_jvp_fixture(poly_roots, ps)
    out["likelihood"] = likelihood_fixture()
    out["parallax"] = parallax_fixture()
    for name, d in out.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print(f"[golden] wrote {len(out)} fixtures in {time.time() - t0:.1f}s")


if __name__ == "__main__":
    main()
