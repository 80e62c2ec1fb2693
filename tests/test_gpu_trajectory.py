"""Annual-parallax trajectory on the GPU (AnnualParallaxTrajectory.compute,
trajectory.py:106-157) and gradients through it.

* w(t) against the reference's own output (tests/golden/parallax.npz) to 1e-13;
* the Jacobian d w / d(u0, t0, tE, piEE, piEN) against central differences of
  the kernel (relative step 1e-6), 1e-6;
* a light-curve loss sum_i c_i mu(w_i) differentiated through the trajectory
  and the extended-source adjoint, against central differences where those are
  stable, 1e-3 (the reference's gradient tolerance)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
C = pytest.importorskip("caustics_gb300")


def eph(d):
    return tuple(d[k] for k in ("t_jpl", "s_e", "s_n", "s_e_dot", "s_n_dot"))


def test_trajectory_vs_reference_fixture(G):
    d = G("parallax")
    traj = C.AnnualParallaxTrajectory(d["t"], ephemeris=eph(d))
    for k in (0, 1):
        u0, t0, tE, piEE, piEN = d[f"params{k}"]
        w = traj.compute(d["t"], u0=u0, t0=t0, tE=tE, piEE=piEE, piEN=piEN)
        assert np.max(np.abs(w - d[f"w{k}"])) < 1e-13
        wp = traj.compute(d["t"], parametrization="polar", u0=u0, t0=t0, tE=tE, piE=np.hypot(piEE, piEN),
                          psi=np.arctan2(piEE, piEN))
        assert np.max(np.abs(wp - d[f"w{k}"])) < 1e-13


def test_trajectory_jacobian():
    rng = np.random.default_rng(3)
    t_jpl = np.arange(0.0, 200.0 + 1, 1.0)
    ph = 2 * np.pi * t_jpl / 365.25
    e = (np.cos(ph), 0.4 * np.sin(ph), -np.sin(ph) * 2 * np.pi / 365.25, 0.4 * np.cos(ph) * 2 * np.pi / 365.25)
    traj = C.AnnualParallaxTrajectory(None, ephemeris=(t_jpl,) + e)
    t = np.sort(rng.uniform(5.0, 195.0, 64))
    theta = np.array([0.12, 101.3, 27.0, 0.31, -0.22])
    w, J = traj.jacobian(t, *theta)
    J = J.cpu().numpy()
    for k in range(5):
        h = 1e-6 * max(abs(theta[k]), 1e-2)
        p, m = theta.copy(), theta.copy()
        p[k] += h
        m[k] -= h
        fd = (traj.jacobian(t, *p)[0] - traj.jacobian(t, *m)[0]).cpu().numpy() / (2 * h)
        assert np.max(np.abs(J[:, k] - fd)) < 1e-6 * max(1.0, np.max(np.abs(fd)))


def test_gradient_through_trajectory_and_contours(G):
    d = G("parallax")
    traj = C.AnnualParallaxTrajectory(d["t"], ephemeris=eph(d))
    t = torch.as_tensor(np.linspace(8180.0, 8220.0, 12), device="cuda")
    lens = torch.tensor([0.9, 0.2, 2e-2, 0.6], dtype=torch.float64, device="cuda")  # s, q, rho, u1
    opts = dict(npts_limb=150, limb_darkening=True, npts_ld=40, precision="fp64")
    c = torch.as_tensor(np.random.default_rng(5).normal(size=12), device="cuda")
    theta0 = np.array([0.05, 8200.3, 25.0, 0.2, -0.15])

    def loss(theta, lens_p):
        names = ("u0", "t0", "tE", "piEE", "piEN")
        w = traj.compute(t, **dict(zip(names, theta)))
        return (C.ExtendedSourceMagnification.apply(w, lens_p, opts) * c).sum()

    th = [torch.tensor(v, dtype=torch.float64, device="cuda", requires_grad=True) for v in theta0]
    lp = lens.clone().requires_grad_(True)
    loss(th, lp).backward()
    g = np.array([float(x.grad) for x in th] + list(lp.grad.cpu().numpy()))

    def f(v):
        return float(loss([torch.tensor(x, dtype=torch.float64, device="cuda") for x in v[:5]],
                          torch.as_tensor(v[5:], device="cuda")))

    v0 = np.concatenate([theta0, lens.cpu().numpy()])
    checked = 0
    for k in range(len(v0)):
        h = 1e-7 * max(abs(v0[k]), 1e-2)
        est = []
        for step in (h, 2 * h):
            p, m = v0.copy(), v0.copy()
            p[k] += step
            m[k] -= step
            est.append((f(p) - f(m)) / (2 * step))
        if abs(est[0] - est[1]) > 1e-4 * max(abs(est[0]), 1e-6):
            continue
        assert abs(g[k] - est[0]) <= 1e-3 * max(abs(est[0]), 1e-2), (k, g[k], est)
        checked += 1
    assert checked >= 6
