"""The C ABI as torch operators (caustics_gb300/ops.py): registration and
shape functions without a GPU; on the GPU, torch.compile(fullgraph=True) over
the ops with back-propagation through the hand-written adjoints, against eager
execution and the Python API (the reference registers its solver as XLA
custom calls, src/caustics/ehrlich_aberth_primitive.py:15-28, :359-373).
The compiled graphs use the aot_eager backend: it runs dynamo's capture and
AOTAutograd (where the fake and autograd registrations are exercised) without
generating kernels of its own."""
import numpy as np
import pytest
import torch

import caustics_gb300  # noqa: F401  (registers torch.ops.caustics)

OPS = ("ea_solve", "ea_roots_vjp", "mag_point_source", "mag_extended_source", "mag_extended_source_grad", "mag",
       "mag_lc_batched", "mag_lc_batched_vjp")


def test_ops_registered():
    for name in OPS:
        assert hasattr(torch.ops.caustics, name), name


def test_fake_shapes():
    from torch._subclasses.fake_tensor import FakeTensorMode
    with FakeTensorMode():
        off = torch.empty(4, dtype=torch.int64, device="cuda")
        t = torch.empty(300, dtype=torch.float64, device="cuda")
        cv = torch.empty(3, 8, dtype=torch.float64, device="cuda")
        assert torch.ops.caustics.mag_lc_batched(off, t, cv, 200, True, 100, 2500, 1).shape == (300,)
        cot = torch.empty(300, dtype=torch.float64, device="cuda")
        assert torch.ops.caustics.mag_lc_batched_vjp(off, t, cv, cot, 200, True, 100, 2500, 1).shape == (3, 8)
        c = torch.empty(7, 11, dtype=torch.complex128, device="cuda")
        assert torch.ops.caustics.ea_solve(c, None, 100, 0).shape == (7, 10)
        w = torch.empty(5, dtype=torch.complex128, device="cuda")
        p = torch.empty(4, dtype=torch.float64, device="cuda")
        m, g = torch.ops.caustics.mag_extended_source_grad(w, p, 100, True, 50, 2500, 1)
        assert m.shape == (5,) and g.shape == (5, 6)
        assert torch.ops.caustics.mag(w, 1e-2, 2, 1.0, 0.1, 0.0, 0.0, 0.0, 100, True, 0.5, 50, 2500, 1).dtype == \
            torch.float64


def _curves():
    t = np.concatenate([np.linspace(-0.3, 0.3, 9), np.linspace(-1.0, 1.0, 7)])
    off = np.array([0, 9, 16], dtype=np.int64)
    cv = np.array([[1.1, 5e-3, 1e-2, 0.5, 0.05, 0.6, 0.0, 20.0],
                   [0.95, 0.3, 2e-2, 0.4, 0.08, 1.2, 0.1, 1.0]])
    return off, t, cv


@pytest.mark.gpu
def test_compiled_light_curve_and_backward_match_eager():
    off, t, cv = _curves()
    dev = torch.device("cuda", 0)
    offd, td = torch.as_tensor(off, device=dev), torch.as_tensor(t, device=dev)
    cot = torch.as_tensor(np.random.default_rng(4).normal(size=len(t)), device=dev)

    def loss(curves):
        m = torch.ops.caustics.mag_lc_batched(offd, td, curves, 100, True, 50, 2500, 1)
        return (m * cot).sum(), m

    c_eager = torch.as_tensor(cv, device=dev).requires_grad_(True)
    l_e, m_e = loss(c_eager)
    l_e.backward()
    compiled = torch.compile(loss, fullgraph=True, backend="aot_eager")
    c_comp = torch.as_tensor(cv, device=dev).requires_grad_(True)
    l_c, m_c = compiled(c_comp)
    l_c.backward()
    # every sum runs in a fixed order, so eager and compiled give identical bits
    assert torch.equal(m_c, m_e)
    assert torch.equal(c_comp.grad, c_eager.grad)
    g_api, _ = caustics_gb300.mag_lc_batched_vjp(off, t, cv, cot.cpu().numpy(), npts_limb=100, limb_darkening=True,
                                                 npts_ld=50, precision="mixed")
    assert torch.equal(c_eager.grad, g_api)


@pytest.mark.gpu
def test_compiled_extended_source_gradients():
    dev = torch.device("cuda", 0)
    w = torch.tensor([0.02 + 0.01j, -0.1 + 0.05j], dtype=torch.complex128, device=dev)
    p = torch.tensor([1.1, 5e-3, 1e-2, 0.5], dtype=torch.float64, device=dev)

    def f(w, p):
        return torch.ops.caustics.mag_extended_source(w, p, 2, 100, True, 50, 2500, 0).sum()

    w1, p1 = w.clone().requires_grad_(True), p.clone().requires_grad_(True)
    f(w1, p1).backward()
    w2, p2 = w.clone().requires_grad_(True), p.clone().requires_grad_(True)
    torch.compile(f, fullgraph=True, backend="aot_eager")(w2, p2).backward()
    m, g = caustics_gb300.mag_extended_source_grad(w, 1e-2, npts_limb=100, limb_darkening=True, u1=0.5, npts_ld=50,
                                                   s=1.1, q=5e-3, precision="fp64")
    for gw, gp in ((w1.grad, p1.grad), (w2.grad, p2.grad)):
        assert torch.allclose(gp, g[:, :4].sum(0), rtol=1e-12)
        assert torch.allclose(gw, torch.complex(g[:, 4], g[:, 5]), rtol=1e-12)


@pytest.mark.gpu
def test_compiled_root_solver_gradient():
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(9)
    c = torch.as_tensor(rng.normal(size=(16, 6)) + 1j * rng.normal(size=(16, 6)), device=dev)

    def f(c):
        z = torch.ops.caustics.ea_solve(c, None, 2500, 0)
        return (z.real ** 2 + 0.3 * z.imag).sum()

    c1, c2 = c.clone().requires_grad_(True), c.clone().requires_grad_(True)
    f(c1).backward()
    torch.compile(f, fullgraph=True, backend="aot_eager")(c2).backward()
    assert torch.allclose(c1.grad, c2.grad, rtol=1e-12)
    # against central differences along a random direction (torch's convention:
    # the directional derivative along d is Re(conj(grad) d))
    d = torch.as_tensor(rng.normal(size=(16, 6)) + 1j * rng.normal(size=(16, 6)), device=dev)
    h = 1e-7
    fd = (f(c + h * d) - f(c - h * d)) / (2 * h)
    ad = (c1.grad.conj() * d).real.sum()
    assert abs(float(fd - ad)) < 1e-5 * max(1.0, abs(float(fd)))


@pytest.mark.gpu
def test_opcheck_light_curve():
    off, t, cv = _curves()
    dev = torch.device("cuda", 0)
    args = (torch.as_tensor(off, device=dev), torch.as_tensor(t, device=dev),
            torch.as_tensor(cv, device=dev).requires_grad_(True), 100, True, 50, 2500, 1)
    torch.library.opcheck(torch.ops.caustics.mag_lc_batched.default, args,
                          test_utils=("test_schema", "test_autograd_registration", "test_faketensor"))
