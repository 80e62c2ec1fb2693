"""Critical curves and caustics on the GPU (critical_and_caustic_curves,
point_source.py:1582-1649).

* against the reference's own output (tests/golden/caustics_binary.npz): the
  set of critical / caustic points at every phase to 1e-10 (the labels of the
  first phase's complex-conjugate pair at phi = -pi depend on last-bit
  rounding of its nearly real coefficients, so curves are compared per phase);
* against the oracle's chaining: the same curves up to a relabelling, 1e-10;
* size-independent properties at 10^4 phases: det J = 0 on every critical
  point, caustic = lens_eq(critical), curves continuous."""
import numpy as np
import pytest

from oracle import caustics_oracle as O

pytestmark = pytest.mark.gpu
C = pytest.importorskip("caustics_gb300")


def setdist(a, b):
    return max(np.max(np.min(np.abs(a[:, None] - b[None, :]), axis=1)),
               np.max(np.min(np.abs(b[:, None] - a[None, :]), axis=1)))


def relabel(a, b):
    """Rows of b reordered to match rows of a at the first phase."""
    return b[[int(np.argmin(np.abs(b[:, 0] - a[i, 0]))) for i in range(a.shape[0])]]


def test_binary_vs_reference_fixture(G):
    d = G("caustics_binary")
    zcr, zca = C.critical_and_caustic_curves(npts=int(d["npts"]), s=float(d["s"]), q=float(d["q"]))
    assert zcr.shape == d["z_cr"].shape
    for k in range(zcr.shape[1]):
        assert setdist(zcr[:, k], d["z_cr"][:, k]) < 1e-10
        assert setdist(zca[:, k], d["z_ca"][:, k]) < 1e-10


@pytest.mark.parametrize("nlenses,params", [(2, dict(s=0.9, q=0.2)), (2, dict(s=1.1, q=5e-3)),
                                            (2, dict(s=2.5, q=1.0)),
                                            (3, dict(s=1.0, q=0.5, q3=0.3, r3=0.9, psi=1.1)),
                                            (3, dict(s=0.8, q=0.8, q3=0.1, r3=1.3, psi=2.0))])
def test_chains_match_the_oracle(nlenses, params):
    zcr, zca = C.critical_and_caustic_curves(npts=300, nlenses=nlenses, **params)
    ocr, oca = O.critical_and_caustic_curves(npts=300, nlenses=nlenses, **params)
    order = [int(np.argmin(np.abs(ocr[:, 0] - zcr[i, 0]))) for i in range(zcr.shape[0])]
    assert sorted(order) == list(range(zcr.shape[0]))
    assert np.max(np.abs(zcr - ocr[order])) < 1e-10
    assert np.max(np.abs(zca - oca[order])) < 1e-10


@pytest.mark.parametrize("nlenses,params", [(2, dict(s=1.1, q=5e-3)), (3, dict(s=1.0, q=0.5, q3=0.3, r3=0.9, psi=1.1))])
def test_properties_at_scale(nlenses, params):
    zcr, zca = C.critical_and_caustic_curves(npts=10000, nlenses=nlenses, **params)
    lens = O._lens_from_params(nlenses, params)
    z = zcr + lens.x_cm
    assert np.max(np.abs(O.lens_eq_det_jac(z, lens))) < 1e-9
    assert np.max(np.abs(O.lens_eq(z, lens) - lens.x_cm - zca)) < 1e-12
    step = np.abs(np.diff(zcr, axis=1))
    assert np.max(step) < 0.05  # no jumps between curves (typical step ~1e-3)


def test_single_lens_and_arguments():
    zcr, zca = C.critical_and_caustic_curves(npts=64, nlenses=1)
    assert np.allclose(np.abs(zcr), 1.0) and np.all(zca == 0)
    with pytest.raises(C._lib.CausticsError):
        C.critical_and_caustic_curves(npts=1, s=1.0, q=0.5)
