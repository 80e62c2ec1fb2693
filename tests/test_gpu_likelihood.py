"""Marginalised log-likelihood on the GPU (marginalized_log_likelihood,
linalg.py:10-94, diagonal covariance), its gradient with respect to the
magnifications, and the likelihood's gradient with respect to the light-curve
parameters through LightCurveLogLikelihood.

Tolerances: beta and ll 1e-11 relative against the reference's fixture (the
2x2 solve is closed-form here, linalg.solve there); d ll / d A 1e-10 against
the oracle's closed form; curve-parameter gradients 1e-3 against central
differences where those are stable (as for the light-curve VJP)."""
import numpy as np
import pytest
import torch

from oracle import caustics_oracle as O

pytestmark = pytest.mark.gpu
C = pytest.importorskip("caustics_gb300")


def test_batched_vs_reference_fixture(G):
    d = G("likelihood")
    beta, ll, g = C.marginalized_log_likelihood_batched(d["offsets"], d["A"], d["fobs"], d["C_inv"],
                                                        return_grad=True)
    assert np.max(np.abs(beta - d["beta"]) / np.abs(d["beta"])) < 1e-11
    assert np.max(np.abs(ll - d["ll_each"]) / np.abs(d["ll_each"])) < 1e-11
    off = d["offsets"]
    for k in range(len(off) - 1):
        s = slice(off[k], off[k + 1])
        a, f, c = d["A"][s], d["fobs"][s], d["C_inv"][s]
        M = np.stack([a, np.ones_like(a)], axis=1)
        Sig = np.linalg.inv(M.T @ (c[:, None] * M))
        ref = O.marginalized_log_likelihood_grad(a, f, c, d["beta"][k], Sig)
        assert np.max(np.abs(g[s] - ref)) < 1e-10 * np.max(np.abs(ref))


def test_list_api_returns_the_sum(G):
    d = G("likelihood")
    off = d["offsets"]
    sl = [slice(off[i], off[i + 1]) for i in range(len(off) - 1)]
    betas, ll = C.marginalized_log_likelihood([d["A"][s] for s in sl], [d["fobs"][s] for s in sl],
                                              [d["C_inv"][s] for s in sl])
    assert abs(ll - d["ll"]) < 1e-11 * abs(d["ll"])
    assert np.allclose(np.stack(betas), d["beta"], rtol=1e-11, atol=0)
    with pytest.raises(NotImplementedError):
        C.marginalized_log_likelihood([d["A"]], [d["fobs"]], [d["C_inv"]], dense_covariance=True)


def test_singular_and_empty_curves():
    off = np.array([0, 0, 1, 4, 8])
    A = np.array([2.0, 3.0, 3.0, 3.0, 1.0, 2.0, 3.0, 4.0])
    f = 2 * A + 1
    c = np.ones(8)
    beta, ll = C.marginalized_log_likelihood_batched(off, A, f, c)
    assert np.all(np.isnan(ll[:3])) and np.isfinite(ll[3])
    assert np.allclose(beta[3], [2.0, 1.0])


def test_likelihood_gradient_through_light_curves():
    rng = np.random.default_rng(8)
    ncur, m = 3, 10
    cv = np.stack([10 ** rng.uniform(np.log10(0.5), np.log10(2), ncur), 10 ** rng.uniform(-2, 0, ncur),
                   10 ** rng.uniform(-2.5, -1.5, ncur), rng.uniform(0.2, 0.8, ncur), rng.uniform(-0.3, 0.3, ncur),
                   rng.uniform(0, 2 * np.pi, ncur), np.zeros(ncur), 10 ** rng.uniform(1, 1.5, ncur)], axis=1)
    off = torch.as_tensor(np.arange(ncur + 1) * m, device="cuda")
    t = torch.as_tensor(np.concatenate([np.sort(rng.uniform(-1.5 * te, 1.5 * te, m)) for te in cv[:, 7]]), device="cuda")
    opts = dict(npts_limb=100, limb_darkening=True, npts_ld=40, precision="fp64")
    mag = C.mag_lc_batched(off, t, torch.as_tensor(cv, device="cuda"), **{k: v for k, v in opts.items()})
    fobs = 1.5 * mag + 0.3 + 0.01 * torch.randn_like(mag)
    cinv = torch.full_like(mag, 1e4)
    curves = torch.tensor(cv, device="cuda", requires_grad=True)
    ll = C.LightCurveLogLikelihood.apply(curves, off, t, fobs, cinv, opts)
    w = torch.tensor([1.0, -0.5, 2.0], dtype=torch.float64, device="cuda")
    (ll * w).sum().backward()
    g = curves.grad.cpu().numpy()

    def f(cvv):
        l = C.LightCurveLogLikelihood.apply(torch.as_tensor(cvv, device="cuda"), off, t, fobs, cinv, opts)
        return float((l * w).sum())

    checked = 0
    for ci in range(ncur):
        for k in range(8):
            h = 1e-7 * max(abs(cv[ci, k]), 1e-2 if k in (4, 5, 6) else 1e-3)
            est = []
            for step in (h, 2 * h):
                p, q = cv.copy(), cv.copy()
                p[ci, k] += step
                q[ci, k] -= step
                est.append((f(p) - f(q)) / (2 * step))
            if abs(est[0] - est[1]) > 1e-4 * max(abs(est[0]), 1e-6):
                continue
            assert abs(g[ci, k] - est[0]) <= 1e-3 * max(abs(est[0]), 1e-2), (ci, k, g[ci, k], est)
            checked += 1
    assert checked >= 12
