"""Host checks of the FP32 Gaspari-Cohn form the mixed-precision analyses use.

For 1 <= z < 2 the published fifth-order function (Gaspari and Cohn 1999,
eq. 4.10) vanishes to fourth order at z = 2, and the polynomial form cancels
there in FP32.  The device's FP32 branch evaluates the exact factored form
z f(z) = (2 - z)^4 (z^2 + 2z - 1/2) / 12; FP64 keeps the polynomial, whose
operation order the oracle shares."""
from fractions import Fraction

import numpy as np


def _poly(z):
    return ((((z / 12 - Fraction(1, 2)) * z + Fraction(5, 8)) * z + Fraction(5, 3)) * z - 5) * z + 4 - Fraction(2, 3) / z


def _factored(z):
    return (2 - z) ** 4 * (z * z + 2 * z - Fraction(1, 2)) / (12 * z)


def test_factored_form_is_the_polynomial_exactly():
    for i in range(0, 201):
        z = 1 + Fraction(i, 200)
        assert _poly(z) == _factored(z)
    assert _poly(Fraction(2)) == 0


def test_fp32_factored_form_positive_inside_the_support_and_accurate():
    z = np.linspace(1.0, 2.0, 400_001)[:-1]
    z32 = z.astype(np.float32)
    t = np.float32(2) - z32
    f32 = (t * t) * (t * t) * ((z32 + np.float32(2)) * z32 - np.float32(0.5)) / (np.float32(12) * z32)
    assert (f32 > 0).all()
    zz = z32.astype(np.float64)  # the FP32 argument, widened
    ref = ((((zz / 12 - 0.5) * zz + 0.625) * zz + 5.0 / 3.0) * zz - 5.0) * zz + 4.0 - 2.0 / (3.0 * zz)
    big = ref > 1e-6
    assert np.max(np.abs(f32[big] - ref[big]) / ref[big]) < 1e-5
    # the FP32 polynomial does not stay positive near the support's edge
    p32 = ((((z32 / np.float32(12) - np.float32(0.5)) * z32 + np.float32(0.625)) * z32 + np.float32(5 / 3)) * z32
           - np.float32(5)) * z32 + np.float32(4) - np.float32(2) / (np.float32(3) * z32)
    assert (p32 <= 0).sum() > 1000
