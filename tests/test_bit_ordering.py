"""The contour kernel compares squared distances and interval lengths by their
IEEE-754 bit patterns on the integer pipe (step maps, the refinement's
labelling and gap ranking).  That rests on one property, checked here on the
CPU: for doubles >= +0 (zero, subnormals, normals, +inf) the bit patterns read
as unsigned 64-bit integers order exactly as the values do, and every NaN,
of either sign, reads above +inf, so a NaN never becomes a nearest root."""
import numpy as np


def test_nonnegative_doubles_order_as_unsigned_bit_patterns():
    rng = np.random.default_rng(0)
    v = np.concatenate([np.abs(rng.standard_normal(20000)) * 10.0 ** rng.integers(-300, 300, 20000),
                        [0.0, 5e-324, 2.2250738585072014e-308, 1.0, np.finfo(np.float64).max, np.inf],
                        np.abs(rng.standard_normal(1000)) * 1e-310])
    u = v.view(np.uint64)
    order_v = np.argsort(v, kind="stable")
    us = u[order_v]
    assert np.all(us[1:] >= us[:-1])
    a, b = rng.choice(v, 50000), rng.choice(v, 50000)
    assert np.array_equal(a < b, a.view(np.uint64) < b.view(np.uint64))


def test_every_nan_reads_above_infinity():
    inf_bits = np.array([np.inf]).view(np.uint64)[0]
    nans = np.array([np.nan, -np.nan]).view(np.uint64)
    nans = np.concatenate([nans, np.array([0x7FF0000000000001, 0xFFF0000000000001, 0xFFFFFFFFFFFFFFFF],
                                          dtype=np.uint64)])
    assert np.all(np.isnan(nans.view(np.float64)))
    assert np.all(nans > inf_bits)
