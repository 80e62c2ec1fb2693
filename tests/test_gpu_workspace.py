"""The workspace forms of the single-evaluation entry points
(cgb_mag_extended_source_ws, cgb_mag_extended_source_grad_ws, cgb_mag_ws),
which the Python functions call, against the plain forms: a separate kernel
orders each first limb point ahead of the contour kernel instead of a lane
group inside it, with the same reference-arithmetic iteration, so the results
are identical bit for bit.  Also the refusals of a short or missing
workspace."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
C = pytest.importorskip("caustics_gb300")
from caustics_gb300 import _lib as L  # noqa: E402
from caustics_gb300 import api as A  # noqa: E402

P = lambda x: ctypes.c_void_p(x.data_ptr())


def sources(n, seed):
    rng = np.random.default_rng(seed)
    w = rng.uniform(-0.6, 0.6, n) + 1j * rng.uniform(-0.6, 0.6, n)
    return torch.as_tensor(w, device="cuda")


LENSES = [(2, dict(s=0.9, q=0.1)), (2, dict(s=1.1, q=5e-3)), (3, dict(s=1.2, q=0.3, q3=0.02, r3=0.8, psi=1.1))]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("nl,lens", LENSES)
def test_extended_source_workspace_form_equals_plain(precision, nl, lens):
    w = sources(300, 3)
    kw = dict(npts_limb=100, limb_darkening=True, u1=0.5, npts_ld=40, precision=precision)
    got = C.mag_extended_source(w, 1e-2, nlenses=nl, **kw, **lens)
    opts = A._es_options(100, True, 0.5, 40, 2500, precision)
    mag = torch.empty(300, dtype=torch.float64, device="cuda")
    st = torch.zeros(300, dtype=torch.int32, device="cuda")
    rc = L.lib().cgb_mag_extended_source(P(w), P(mag), 300, 1e-2, L.lens_params(nl, lens), opts, P(st),
                                         A._stream())
    assert rc == 0, L.lib().cgb_last_error()
    assert torch.equal(got, mag)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_mag_and_grad_workspace_forms_equal_plain(precision):
    lens = dict(s=0.9, q=0.1)
    w = sources(300, 4)
    opts = A._es_options(100, True, 0.5, 40, 2500, precision)
    got, route = C.mag(w, 1e-2, npts_limb=100, limb_darkening=True, u1=0.5, npts_ld=40, precision=precision,
                       return_route=True, **lens)
    mag = torch.empty(300, dtype=torch.float64, device="cuda")
    rt = torch.empty(300, dtype=torch.uint8, device="cuda")
    rc = L.lib().cgb_mag(P(w), P(mag), P(rt), 300, 1e-2, L.lens_params(2, lens), opts, None, A._stream())
    assert rc == 0, L.lib().cgb_last_error()
    assert torch.equal(got, mag) and torch.equal(route, rt.bool())
    gm, gg = C.mag_extended_source_grad(w, 1e-2, npts_limb=100, limb_darkening=True, u1=0.5, npts_ld=40,
                                        precision=precision, **lens)
    mag2 = torch.empty(300, dtype=torch.float64, device="cuda")
    g = torch.empty((300, 6), dtype=torch.float64, device="cuda")
    rc = L.lib().cgb_mag_extended_source_grad(P(w), P(mag2), P(g), 300, 1e-2, L.lens_params(2, lens), opts, None,
                                              A._stream())
    assert rc == 0, L.lib().cgb_last_error()
    assert torch.equal(gm, mag2) and torch.equal(gg, g)


def test_workspace_refusals():
    lib = L.lib()
    assert lib.cgb_mag_extended_source_workspace_bytes(1000) == 8000
    assert lib.cgb_mag_extended_source_workspace_bytes(0) == 0
    w = sources(10, 5)
    mag = torch.empty(10, dtype=torch.float64, device="cuda")
    ws = torch.empty(10, dtype=torch.int64, device="cuda")
    opts = A._es_options(100, False, 0.0, 40, 2500, "mixed")
    lp = L.lens_params(2, dict(s=0.9, q=0.1))
    assert lib.cgb_mag_extended_source_ws(P(w), P(mag), 10, 1e-2, lp, opts, None, None, 0, None) == L.CGB_ERR_INVALID
    assert lib.cgb_mag_extended_source_ws(P(w), P(mag), 10, 1e-2, lp, opts, None, P(ws), 79, None) == \
        L.CGB_ERR_INVALID
    misaligned = ctypes.c_void_p(ws.data_ptr() + 4)
    assert lib.cgb_mag_extended_source_ws(P(w), P(mag), 10, 1e-2, lp, opts, None, misaligned, 80, None) == \
        L.CGB_ERR_INVALID
    assert lib.cgb_mag_extended_source_ws(None, None, 0, 1e-2, lp, opts, None, None, 0, None) == 0
