"""Derivatives of the root-solver primitive on the GPU: the implicit-function
JVP dz_r = -sum_k z_r^k dp_k / p'(z_r) (ehrlich_aberth_primitive.py:252-312),
its transpose / conjugate transpose, and torch autograd through poly_roots.

Known answer: central differences of the reference solver's roots
(tests/golden/roots_jvp.npz): 1e-7 relative for degree 5, 1e-5 for degree 10
(one nearly paired root pair limits the difference quotient there); against the
oracle's restatement of the same rule: 1e-10."""
import numpy as np
import pytest
import torch

from oracle import caustics_oracle as O

pytestmark = pytest.mark.gpu
C = pytest.importorskip("caustics_gb300")


@pytest.mark.parametrize("deg,tol", [("5", 1e-7), ("10", 1e-5)])
def test_jvp_known_answer(G, deg, tol):
    d = G("roots_jvp")
    p, z, dp = d["p" + deg], d["z" + deg], d["dp" + deg]
    dz = C.roots_jvp(p, z, dp)
    assert np.max(np.abs(dz - d["dz" + deg]) / np.abs(d["dz" + deg])) < tol
    ref = O.roots_jvp(p, z, dp)
    assert np.max(np.abs(dz - ref) / np.abs(ref)) < 1e-10


@pytest.mark.parametrize("deg", ["5", "10"])
def test_vjp_is_the_transpose(G, deg):
    d = G("roots_jvp")
    p, z, dp = (torch.as_tensor(d[k + deg], device="cuda") for k in ("p", "z", "dp"))
    rng = np.random.default_rng(0)
    ct = torch.as_tensor(rng.normal(size=z.shape) + 1j * rng.normal(size=z.shape), device="cuda")
    jdp = C.roots_jvp(p, z, dp)
    lhs = (ct * jdp).sum()
    rhs = (C.roots_vjp(p, z, ct) * dp).sum()
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)
    lhs_h = (ct.conj() * jdp).sum()
    rhs_h = (C.roots_vjp(p, z, ct, conjugate=True).conj() * dp).sum()
    assert abs(lhs_h - rhs_h) < 1e-10 * abs(lhs_h)


def test_autograd_through_poly_roots(G):
    """loss = Re sum conj(a) z(p); torch's gradient g satisfies
    d loss = Re sum conj(g) dp for every tangent dp."""
    d = G("roots_jvp")
    p_lo = torch.as_tensor(d["p5"], device="cuda")
    c = p_lo.flip(-1).clone().requires_grad_(True)  # highest order first, as poly_roots takes them
    z = C.poly_roots(c, itmax=2500)
    rng = np.random.default_rng(1)
    a = torch.as_tensor(rng.normal(size=z.shape) + 1j * rng.normal(size=z.shape), device="cuda")
    (a.conj() * z).real.sum().backward()
    dp_lo = torch.as_tensor(d["dp5"], device="cuda")
    pred = (c.grad.conj() * dp_lo.flip(-1)).real.sum()
    exact = (a.conj() * C.roots_jvp(p_lo, z.detach(), dp_lo)).real.sum()
    assert abs(pred - exact) < 1e-10 * abs(exact)


def test_invalid_and_empty():
    z = torch.zeros((0, 5), dtype=torch.complex128, device="cuda")
    p = torch.zeros((0, 6), dtype=torch.complex128, device="cuda")
    assert C.roots_jvp(p, z, p).shape == (0, 5)
    with pytest.raises(C._lib.CausticsError):
        C.roots_jvp(torch.zeros((2, 1), dtype=torch.complex128, device="cuda"),
                    torch.zeros((2, 0), dtype=torch.complex128, device="cuda"),
                    torch.zeros((2, 1), dtype=torch.complex128, device="cuda"))
