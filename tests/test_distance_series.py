"""Host check of the series the geographic search evaluates distances with.

For half chords h <= 0.05 (great-circle distances up to about 640 km) the
device computes asin(h) by its Maclaurin series through h^11, in FP64
multiply-adds; the distances it reports must agree with the host's asin to
the tolerance the parity tests use (1e-13 relative), and in fact to a few
units in the last place."""
import math

import numpy as np


def _series(h):
    h2 = h * h
    q = 63.0 / 2816.0
    for c in (35.0 / 1152.0, 5.0 / 112.0, 3.0 / 40.0, 1.0 / 6.0):
        q = q * h2 + c
    return h + (h * h2) * q


def test_coefficients_are_the_maclaurin_series():
    for n, c in enumerate((1.0, 1.0 / 6.0, 3.0 / 40.0, 5.0 / 112.0, 35.0 / 1152.0, 63.0 / 2816.0)):
        assert c == math.factorial(2 * n) / (4 ** n * math.factorial(n) ** 2 * (2 * n + 1))


def test_series_matches_asin_on_short_chords():
    h = np.concatenate([np.linspace(0.0, 0.05, 200_001)[1:], np.geomspace(1e-12, 0.05, 2_000)])
    got = _series(h)
    want = np.array([math.asin(x) for x in h])
    rel = np.abs(got - want) / want
    assert rel.max() < 4e-16
