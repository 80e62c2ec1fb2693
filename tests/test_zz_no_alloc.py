"""cgb_mag_lc_batched_noalloc: the batched light-curve entry point with its
queue in the library's static device array instead of a caller workspace.
Compared with cgb_mag_lc_batched on the same curves, on two calls in a row (the
second reuses the static queue), to 1e-12 relative: same kernels, same launch
shape.  Placed last in collection order; passes alone and after the others."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
C = pytest.importorskip("caustics_gb300")
from caustics_gb300 import _lib as L  # noqa: E402

OPTS = dict(npts_limb=100, limb_darkening=True, npts_ld=40)


def curves(seed, ncurves=5):
    rng = np.random.default_rng(seed)
    lens = rng.integers(20, 60, ncurves)
    cv = np.stack([10 ** rng.uniform(np.log10(0.3), np.log10(3), ncurves), 10 ** rng.uniform(-4, 0, ncurves),
                   10 ** rng.uniform(-3, -1, ncurves), rng.uniform(0.2, 0.8, ncurves), rng.uniform(-0.3, 0.3, ncurves),
                   rng.uniform(0, 2 * np.pi, ncurves), np.zeros(ncurves), 10 ** rng.uniform(np.log10(5), 2, ncurves)],
                  axis=1)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    t = np.concatenate([np.sort(rng.uniform(-2 * te, 2 * te, n)) for te, n in zip(cv[:, 7], lens)])
    return (torch.as_tensor(off, device="cuda"), torch.as_tensor(t, device="cuda"),
            torch.as_tensor(cv, device="cuda"))


def noalloc(off, t, cv, precision, opts_kw=OPTS):
    n = t.numel()
    mag = torch.empty(n, dtype=torch.float64, device="cuda")
    route = torch.empty(n, dtype=torch.uint8, device="cuda")
    opts = L.EsOptions(opts_kw["npts_limb"], 1, 0.0, opts_kw["npts_ld"], 2500, L.PREC_MIXED if precision == "mixed"
                       else L.PREC_FP64, 0, 1, 1)
    p = lambda x: ctypes.c_void_p(x.data_ptr())
    rc = L.lib().cgb_mag_lc_batched_noalloc(p(off), p(t), p(cv), cv.shape[0], n, p(mag), p(route), None,
                                            ctypes.byref(opts),
                                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, L.lib().cgb_last_error()
    return mag, route


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_noalloc_matches_workspace_entry_point(precision):
    off, t, cv = curves(17)
    ref, ref_route = C.mag_lc_batched(off, t, cv, precision=precision, return_route=True, **OPTS)
    for _ in range(2):
        m, route = noalloc(off, t, cv, precision)
        assert torch.equal(route.bool(), ref_route)
        assert float((torch.abs(m - ref) / ref).max()) < 1e-12


def test_noalloc_rejects_sizes_beyond_its_scratch():
    opts = L.EsOptions(100, 1, 0.0, 40, 2500, L.PREC_MIXED, 0, 1, 1)
    rc = L.lib().cgb_mag_lc_batched_noalloc(None, None, None, 1, (1 << 18) + 1, None, None, None, ctypes.byref(opts),
                                            None)
    assert rc == L.CGB_ERR_UNSUPPORTED
    assert b"262144" in L.lib().cgb_last_error()


def test_noalloc_beyond_the_row_order_region():
    """140,200 points: above 131,072 the static array holds only the queue and
    the contour kernel orders each first limb point itself.  Fourteen curves far
    from the caustics (every point hexadecapole-accepted) and one crossing the
    central caustic of a q = 5e-3 lens (every point through the contour
    integral, npts_limb 16)."""
    far = [[1.0, 0.5, 1e-3, 0.5, 1.5, 0.3, 0.0, 1.0]] * 14
    near = [[1.1, 5e-3, 1e-2, 0.5, 0.05, 0.6, 0.0, 20.0]]
    lens = [10000] * 14 + [200]
    t = np.concatenate([np.linspace(-1.0, 1.0, 10000)] * 14 + [np.linspace(-0.5, 0.5, 200)])
    off = torch.as_tensor(np.concatenate([[0], np.cumsum(lens)]), device="cuda")
    t, cv = torch.as_tensor(t, device="cuda"), torch.as_tensor(np.array(far + near), device="cuda")
    kw = dict(npts_limb=16, limb_darkening=True, npts_ld=20)
    ref, ref_route = C.mag_lc_batched(off, t, cv, precision="mixed", return_route=True, **kw)
    assert t.numel() > 131072 and 200 <= int(ref_route.sum()) < 1000
    for _ in range(2):
        m, route = noalloc(off, t, cv, "mixed", kw)
        assert torch.equal(route.bool(), ref_route)
        assert float((torch.abs(m - ref) / ref).max()) < 1e-12


def test_noalloc_zero_points():
    opts = L.EsOptions(100, 1, 0.0, 40, 2500, L.PREC_MIXED, 0, 1, 1)
    off = torch.zeros(2, dtype=torch.int64, device="cuda")
    cv = torch.tensor([[1.1, 5e-3, 1e-2, 0.5, 0.05, 0.6, 0.0, 20.0]], dtype=torch.float64, device="cuda")
    rc = L.lib().cgb_mag_lc_batched_noalloc(ctypes.c_void_p(off.data_ptr()), None, ctypes.c_void_p(cv.data_ptr()), 1,
                                            0, None, None, None, ctypes.byref(opts), None)
    assert rc == L.CGB_OK, L.lib().cgb_last_error()
