"""Per-item status words and error returns, made to happen on the GPU by the
inputs alone (nothing here faults, traps or waits): a solver capped at one
iteration, non-finite inputs, curve parameters out of the domain, a limb too
large for the contour kernel, open-segment linking, an empty work queue, and
bit-identical repeated calls.  The reference prints and asserts on
non-convergence (lib/ehrlich_aberth/ehrlich_aberth.h:144-149) and returns NaN
or garbage for the rest; here every case is a status bit or an error code."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

C = pytest.importorskip("caustics_gb300")
from caustics_gb300 import _lib as L  # noqa: E402

LC = dict(npts_limb=100, limb_darkening=True, npts_ld=50)


def test_itmax_one_sets_noconv_with_finite_output():
    rng = np.random.default_rng(2)
    w = rng.uniform(-1.5, 1.5, 256) + 1j * rng.uniform(-1.5, 1.5, 256)
    for prec in ("fp64", "mixed"):
        m, st = C.mag_point_source(w, s=0.9, q=0.1, roots_itmax=1, precision=prec, return_status=True)
        assert np.all(np.isfinite(m))
        assert np.mean((st & L.ST_NOCONV) != 0) > 0.9
        m2, st2 = C.mag_point_source(w, s=0.9, q=0.1, precision=prec, return_status=True)
        assert not np.any(st2 & L.ST_NOCONV)
    st = torch.zeros(4, dtype=torch.int32, device="cuda")
    c = torch.as_tensor(rng.normal(size=(4, 6)) + 1j * rng.normal(size=(4, 6)), device="cuda")
    z = C.ehrlich_aberth(c, None, itmax=1, status=st)
    assert torch.isfinite(torch.view_as_real(z)).all() and bool(((st & L.ST_NOCONV) != 0).all())


def test_non_finite_inputs_give_nan_and_invalid():
    w = np.array([np.nan + 0.1j, np.inf + 0j, 0.1 + 0.1j, complex(0.3, -np.inf)])
    bad = np.array([True, True, False, True])
    m, st = C.mag_point_source(w, s=0.9, q=0.1, return_status=True)
    assert np.all(np.isnan(m[bad])) and np.all(st[bad] == L.ST_INVALID)
    assert np.isfinite(m[2]) and not (st[2] & L.ST_INVALID)
    m, route, st = C.mag(w, 1e-2, s=0.9, q=0.1, u1=0.5, return_route=True, return_status=True, **LC)
    assert np.all(np.isnan(m[bad])) and np.all(st[bad] == L.ST_INVALID) and not route[bad].any()
    assert np.isfinite(m[2])
    m, st = C.mag_extended_source(w, 1e-2, s=0.9, q=0.1, u1=0.5, return_status=True, **LC)
    assert np.all(np.isnan(m[bad])) and np.all((st[bad] & L.ST_INVALID) != 0) and np.isfinite(m[2])
    _, g = C.mag_extended_source_grad(w, 1e-2, s=0.9, q=0.1, u1=0.5, **LC)
    assert np.all(np.isnan(g[bad])) and np.all(np.isfinite(g[2]))
    # roots of a polynomial with a non-finite coefficient
    c = np.array([[1, 2, 3, 4, 5, 1], [1, np.nan, 3, 4, 5, 1]], dtype=np.complex128)
    st = torch.zeros(2, dtype=torch.int32, device="cuda")
    z = C.ehrlich_aberth(torch.as_tensor(c, device="cuda"), None, itmax=500, status=st).reshape(2, 5)
    assert torch.isfinite(torch.view_as_real(z[0])).all() and torch.isnan(torch.view_as_real(z[1])).all()
    assert st.tolist() == [0, L.ST_INVALID]


def test_batched_curve_out_of_domain():
    """A curve with s <= 0, q <= 0, rho <= 0, tE = 0 or a non-finite parameter
    gives NaN and CGB_ST_INVALID on its own points and no gradient; the other
    curves are unaffected."""
    t = np.linspace(-0.5, 0.5, 8)
    good = [1.1, 5e-3, 1e-2, 0.5, 0.05, 0.6, 0.0, 20.0]
    bads = [[-1.1, 5e-3, 1e-2, 0.5, 0.05, 0.6, 0.0, 20.0], [1.1, 0.0, 1e-2, 0.5, 0.05, 0.6, 0.0, 20.0],
            [1.1, 5e-3, -1e-2, 0.5, 0.05, 0.6, 0.0, 20.0], [1.1, 5e-3, 1e-2, 0.5, 0.05, 0.6, 0.0, 0.0],
            [1.1, 5e-3, 1e-2, np.nan, 0.05, 0.6, 0.0, 20.0]]
    cv = np.array([good] + bads + [good])
    off = np.arange(len(cv) + 1) * len(t)
    tt = np.tile(t, len(cv))
    m, route, st = C.mag_lc_batched(off, tt, cv, precision="mixed", return_route=True, return_status=True, **LC)
    m, route, st = m.cpu().numpy(), route.cpu().numpy(), st.cpu().numpy()
    inner = slice(len(t), len(t) * (len(cv) - 1))
    assert np.all(np.isnan(m[inner])) and np.all(st[inner] == L.ST_INVALID) and not route[inner].any()
    ref = C.mag_lc_batched(np.array([0, len(t)]), t, np.array([good]), precision="mixed", **LC).cpu().numpy()
    assert np.array_equal(m[:len(t)], ref) and np.array_equal(m[-len(t):], ref)
    g, _ = C.mag_lc_batched_vjp(off, tt, cv, np.ones(len(tt)), precision="mixed", **LC)
    g = g.cpu().numpy()
    assert np.all(g[1:-1] == 0) and np.all(np.isfinite(g)) and np.array_equal(g[0], g[-1])


def test_limb_too_large_or_small_is_refused():
    with pytest.raises(L.CausticsError, match="npts_limb"):
        C.mag_extended_source(np.array([0.1 + 0.1j]), 1e-2, npts_limb=20000, s=0.9, q=0.1)
    with pytest.raises(L.CausticsError, match="npts_limb"):
        C.mag_extended_source(np.array([0.1 + 0.1j]), 1e-2, npts_limb=4, s=0.9, q=0.1)


def test_open_linking_sets_merge(G):
    d = G("mag_lc_batched_seed2_flagged")
    n = len(d["t"])
    m, st = C.mag_lc_batched(np.arange(n + 1), d["t"], d["curves"], npts_limb=200, limb_darkening=True, npts_ld=100,
                             precision="fp64", return_status=True)
    merge = (st.cpu().numpy() & L.ST_MERGE) != 0
    assert 0 < merge.sum() < n
    assert np.max(np.abs(m.cpu().numpy()[merge] - d["mag"][merge]) / d["mag"][merge]) < 1e-9


def test_empty_queue_drains():
    """Every point accepted by the hexadecapole: the contour kernel finds an
    empty queue and returns; the magnifications are the hexadecapole's."""
    t = np.linspace(-1.0, 1.0, 64)
    cv = np.array([[1.0, 0.5, 1e-3, 0.5, 1.2, 0.3, 0.0, 1.0]])  # far from the caustics
    m, route = C.mag_lc_batched(np.array([0, len(t)]), t, cv, precision="mixed", return_route=True, **LC)
    assert not route.any() and torch.isfinite(m).all() and bool((m >= 1.0).all())
    ev = C.BatchedLightCurves(np.array([0, len(t)]), t, curves_for_tuning=cv, tune=False, **LC)
    assert torch.equal(ev(cv), m)


def test_repeated_calls_are_bit_identical():
    """Sums over contour points and over a curve's points run in a fixed order:
    two identical calls give identical magnifications and gradients."""
    rng = np.random.default_rng(7)
    t = np.sort(rng.uniform(-1, 1, 40))
    cv = np.array([[1.1, 5e-3, 1e-2, 0.5, 0.05, 0.6, 0.0, 20.0], [0.9, 0.3, 2e-2, 0.4, 0.02, 1.1, 0.0, 1.0]])
    off = np.array([0, 25, 40])
    cot = rng.normal(size=len(t))
    for prec in ("fp64", "mixed"):
        g1, m1 = C.mag_lc_batched_vjp(off, t, cv, cot, precision=prec, **LC)
        g2, m2 = C.mag_lc_batched_vjp(off, t, cv, cot, precision=prec, **LC)
        assert torch.equal(g1, g2) and torch.equal(m1, m2)
        f1 = C.mag_lc_batched(off, t, cv, precision=prec, **LC)
        f2 = C.mag_lc_batched(off, t, cv, precision=prec, **LC)
        assert torch.equal(f1, f2)
        # the adjoint's forward runs in another kernel instantiation (its own
        # instruction scheduling), and in mixed precision it polishes every root
        # to full FP64 accuracy where the forward kernels may stop at ~1e-13
        assert torch.allclose(f1, m1, rtol=1e-12 if prec == "fp64" else 1e-10, atol=0)
    w = rng.uniform(-0.2, 0.2, 16) + 1j * rng.uniform(-0.2, 0.2, 16)
    a = C.mag_extended_source_grad(w, 1e-2, s=1.1, q=5e-3, u1=0.5, precision="mixed", **LC)
    b = C.mag_extended_source_grad(w, 1e-2, s=1.1, q=5e-3, u1=0.5, precision="mixed", **LC)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
