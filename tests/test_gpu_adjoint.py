"""GPU adjoint of the extended-source magnification against central finite
differences of the FP64 forward pass, as the reference checks its gradients
(tests/test_extended_source.py:295-331: jacfwd/jacrev vs approx_fprime, rtol 1e-3).

Near critical curves an image moves by ~h/det J, so relative steps of 1e-6
are already outside the linear regime; the steps used are 1e-7 and 1e-8
(relative) and a difference quotient only counts when both agree to 1e-3 and
the limb angle grid is the same at every evaluated point (the discrete
refinement / linking decisions are piecewise constant, as under autodiff).
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import caustics_oracle as O

pytestmark = pytest.mark.gpu
C = pytest.importorskip("caustics_gb300")
from caustics_gb300 import _lib as L  # noqa: E402

NAMES = ("s", "q", "rho", "u1", "wx", "wy")


def fwd_debug(w, rho, s, q, u1, npts, nld, ld, prec):
    lib = L.lib()
    wt = torch.as_tensor(np.atleast_1d(np.asarray(w, dtype=complex))).cuda()
    n = wt.numel()
    mag = torch.empty(n, dtype=torch.float64, device="cuda")
    rl = lib.cgb_debug_record_len(npts)
    dbg = torch.zeros((n, rl), dtype=torch.float64, device="cuda")
    opts = L.EsOptions(npts, int(ld), u1, nld, 2500, prec, 0)
    rc = lib.cgb_debug_extended_source(ctypes.c_void_p(wt.data_ptr()), ctypes.c_void_p(mag.data_ptr()), n, rho,
                                       L.LensParams(2, s, q, 0, 0, 0), opts, None, ctypes.c_void_p(dbg.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    d = dbg.cpu().numpy()
    return mag.cpu().numpy(), d[:, 63:63 + int(d[0, 0])]


def grad(w, rho, s, q, u1, npts, nld, ld, prec):
    lib = L.lib()
    wt = torch.as_tensor(np.atleast_1d(np.asarray(w, dtype=complex))).cuda()
    n = wt.numel()
    mag = torch.empty(n, dtype=torch.float64, device="cuda")
    g = torch.empty((n, 6), dtype=torch.float64, device="cuda")
    opts = L.EsOptions(npts, int(ld), u1, nld, 2500, prec, 0)
    rc = lib.cgb_mag_extended_source_grad(ctypes.c_void_p(wt.data_ptr()), ctypes.c_void_p(mag.data_ptr()),
                                          ctypes.c_void_p(g.data_ptr()), n, rho, L.LensParams(2, s, q, 0, 0, 0), opts,
                                          None, None)
    assert rc == 0, lib.cgb_last_error()
    torch.cuda.synchronize()
    return mag.cpu().numpy(), g.cpu().numpy()


def fd(w, rho, s, q, u1, npts, nld, ld, k, rel):
    p = dict(w=np.asarray(w, dtype=complex), rho=rho, s=s, q=q, u1=u1)
    base = {"wx": 1.0, "wy": 1.0}.get(NAMES[k], abs([s, q, rho, u1][k]) if k < 4 else 1.0)
    h = rel * max(base, 1e-3)
    out = []
    for sgn in (1, -1):
        pp = dict(p)
        if NAMES[k] == "wx":
            pp["w"] = p["w"] + sgn * h
        elif NAMES[k] == "wy":
            pp["w"] = p["w"] + 1j * sgn * h
        else:
            pp[NAMES[k]] = p[NAMES[k]] + sgn * h
        out.append(fwd_debug(pp["w"], pp["rho"], pp["s"], pp["q"], pp["u1"], npts, nld, ld, 0))
    (mp, tp), (mm, tm) = out
    same = np.array([np.array_equal(a, b) for a, b in zip(tp, tm)])
    return (mp - mm) / (2 * h), same


def fd_stable(w, rho, s, q, u1, npts, nld, ld, k):
    f1, s1 = fd(w, rho, s, q, u1, npts, nld, ld, k, 1e-7)
    f2, s2 = fd(w, rho, s, q, u1, npts, nld, ld, k, 1e-8)
    ok = s1 & s2 & (np.abs(f1 - f2) <= 1e-3 * np.maximum(np.abs(f2), 1e-3))
    return f2, ok


def PSCALE(s, q, rho):
    """Natural scales of (s, q, rho, u1, Re w, Im w)."""
    return np.array([s, q, rho, 1.0, rho, rho])


CASES = [  # (points, rho, s, q, u1, npts_limb, npts_ld, limb darkening)
    ("near caustic, LD", 1e-2, 0.9, 0.2, 0.7, 300, 100, True),
    ("near caustic, uniform", 1e-2, 0.9, 0.2, 0.0, 300, 100, False),
    ("planetary, LD", 1e-2, 1.1, 5e-3, 0.5, 300, 100, True),
]


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_adjoint_vs_central_differences(G, case, prec):
    name, rho, s, q, u1, npts, nld, ld = CASES[case]
    if q < 0.01:
        t = np.linspace(-40, 40, 2000)[880:1120:30] / 20.0
        w = (0.05 * np.cos(0.6) + t * np.sin(0.6)) + 1j * (-0.05 * np.sin(0.6) + t * np.cos(0.6))
    else:
        d = G("mag_es4")
        w = np.concatenate([d["w"][:5], [0.6 + 0.4j]])
    mag, g = grad(w, rho, s, q, u1, npts, nld, ld, prec)
    m64, _ = fwd_debug(w, rho, s, q, u1, npts, nld, ld, 0)
    assert np.max(np.abs(mag - m64) / m64) < 1e-6
    checked = 0
    for k in range(6):
        if k == 3 and not ld:
            assert np.all(g[:, 3] == 0)
            continue
        f, ok = fd_stable(w, rho, s, q, u1, npts, nld, ld, k)
        scale = np.maximum(np.abs(f), 1e-3 * mag)
        # mixed precision differentiates its own forward pass, whose FP32
        # quadrature sits ~1e-8 of mu from FP64's; through the 2 mu / rho term
        # of d mu / d rho (and alike) that allows 1e-6 of mu on the parameter's
        # natural scale (measured: 1.8e-7 at w = 0.6 + 0.4i, where d mu / d rho
        # is 2e4 times smaller than 2 mu / rho)
        floor = 1e-6 * mag / PSCALE(s, q, rho)[k] if prec == 1 else 0.0
        err = np.maximum(np.abs(g[:, k] - f) - floor, 0.0) / scale
        checked += ok.sum()
        assert np.all(err[ok] < 1e-3), (NAMES[k], g[ok, k], f[ok])
    assert checked >= 6 * len(w) // 2


@pytest.mark.parametrize("prec", [0, 1])
def test_adjoint_vs_oracle_frozen_structure(G, prec):
    """Against the oracle's frozen-structure finite differences (the smooth
    function autodiff differentiates).  Limb points within ~1e-7 of a caustic
    keep the difference quotient curved down to steps of 1e-8, so a component
    counts only where the steps 1e-8 and 1e-9 (relative) agree to 5e-4."""
    d = G("mag_es4")
    checked = 0
    for w in d["w"][:3]:
        mag, g = grad(np.array([w]), 1e-2, 0.9, 0.2, 0.7, 300, 100, True, prec)
        r1 = O.frozen_gradient(w, 1e-2, 0.9, 0.2, 300, True, 0.7, 100, rel=1e-8)
        r2 = O.frozen_gradient(w, 1e-2, 0.9, 0.2, 300, True, 0.7, 100, rel=1e-9)
        scale = np.maximum(np.abs(r2), 1e-3 * mag[0])
        ok = np.abs(r1 - r2) <= 5e-4 * scale
        assert np.all(np.abs(g[0] - r2)[ok] / scale[ok] < 2e-3), (g[0], r2, ok)
        checked += ok.sum()
    assert checked >= 12


# ---- triple lenses: d mag / d(s, q, rho, u1, Re w0, Im w0, q3, r3, psi) ----
TRIPLE = dict(s=1.0, q=0.5, q3=0.05, r3=0.9, psi=1.1)  # the triple fixture's system (mag_es_triple)
T_NAMES = ("s", "q", "rho", "u1", "wx", "wy", "q3", "r3", "psi")


def _lens3(p):
    return L.LensParams(3, p["s"], p["q"], p["q3"], p["r3"], p["psi"])


def fwd3(w, rho, p, u1, npts, nld, ld):
    """FP64 forward with the limb angle grid of each point (debug record)."""
    lib = L.lib()
    wt = torch.as_tensor(np.atleast_1d(np.asarray(w, dtype=complex))).cuda()
    n = wt.numel()
    mag = torch.empty(n, dtype=torch.float64, device="cuda")
    dbg = torch.zeros((n, lib.cgb_debug_record_len(npts)), dtype=torch.float64, device="cuda")
    rc = lib.cgb_debug_extended_source(ctypes.c_void_p(wt.data_ptr()), ctypes.c_void_p(mag.data_ptr()), n, rho,
                                       _lens3(p), L.EsOptions(npts, int(ld), u1, nld, 2500, 0, 0), None,
                                       ctypes.c_void_p(dbg.data_ptr()), None)
    assert rc == 0, lib.cgb_last_error()
    d = dbg.cpu().numpy()
    return mag.cpu().numpy(), d[:, 63:63 + int(d[0, 0])]


def grad3(w, rho, p, u1, npts, nld, ld, prec):
    m, g = C.mag_extended_source_grad(np.asarray(w, dtype=complex), rho, nlenses=3, npts_limb=npts,
                                      limb_darkening=ld, u1=u1, npts_ld=nld, precision=("fp64", "mixed")[prec], **p)
    return m, g


def fd3_stable(w, rho, p, u1, npts, nld, ld, k):
    """Central differences at relative steps 1e-7 and 1e-8 (absolute for the
    source position and psi), trusted where both agree and every evaluated limb
    grid is the same."""
    res = []
    for rel in (1e-7, 1e-8):
        name = T_NAMES[k]
        vals = dict(p, rho=rho, u1=u1)
        h = rel * (1.0 if name in ("wx", "wy", "psi") else max(abs(vals[name]), 1e-3))
        out = []
        for sgn in (1, -1):
            pp, ww, r, uu = dict(p), np.asarray(w, dtype=complex), rho, u1
            if name == "wx":
                ww = ww + sgn * h
            elif name == "wy":
                ww = ww + 1j * sgn * h
            elif name == "rho":
                r = rho + sgn * h
            elif name == "u1":
                uu = u1 + sgn * h
            else:
                pp[name] = p[name] + sgn * h
            out.append(fwd3(ww, r, pp, uu, npts, nld, ld))
        (mp, tp), (mm, tm) = out
        same = np.array([np.array_equal(a, b) for a, b in zip(tp, tm)])
        res.append(((mp - mm) / (2 * h), same))
    (f1, s1), (f2, s2) = res
    return f2, s1 & s2 & (np.abs(f1 - f2) <= 1e-3 * np.maximum(np.abs(f2), 1e-3))


@pytest.mark.parametrize("ld", [False, True])
@pytest.mark.parametrize("prec", [0, 1])
def test_triple_adjoint_vs_central_differences(G, prec, ld):
    d = G("mag_es_triple")
    w, rho, npts = d["w"], float(d["rho"]), int(d["npts_limb"])
    u1 = 0.6 if ld else 0.0
    mag, g = grad3(w, rho, TRIPLE, u1, npts, 60, ld, prec)
    assert g.shape == (len(w), 9)
    if not ld:
        assert np.max(np.abs(mag - d["mag"]) / d["mag"]) < (1e-9 if prec == 0 else 1e-4)
        assert np.all(g[:, 3] == 0)
    checked = 0
    for k in range(9):
        if k == 3 and not ld:
            continue
        f, ok = fd3_stable(w, rho, TRIPLE, u1, npts, 60, ld, k)
        # a derivative's natural scale is mu / (its parameter's scale): the mixed
        # quadrature's FP32 nodes leave ~1e-7 mu on mu itself
        pscale = (TRIPLE["s"], TRIPLE["q"], rho, 1.0, rho, rho, TRIPLE["q3"], TRIPLE["r3"], 1.0)[k]
        scale = np.maximum(np.abs(f), 1e-3 * mag / pscale)
        err = np.abs(g[:, k] - f) / scale
        checked += ok.sum()
        assert np.all(err[ok] < 1e-3), (T_NAMES[k], g[ok, k], f[ok])
    assert checked >= 8 * len(w) // 2
