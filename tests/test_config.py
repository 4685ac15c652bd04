"""Host checks of configuration numbers (no GPU).  The reference keeps a
config float as `float` (ConfigValue::asFloat, src/framework/adapters/common/
utils/config/ConfigValue.hpp:108) and its policies widen it to double
(LETKF.hpp:52-53), so an inflation of 1.1 acts as 1.100000023841858; the
policy mirror reads every float key that way, and a missing key raises."""
import numpy as np
import pytest

from metada_gb300 import algorithms as alg
from metada_gb300 import synthetic as syn


@pytest.mark.parametrize("x", [1.1, 1.05, 0.1, 500.0, 6.5, 1e-3, 123456.789])
def test_config_floats_are_rounded_to_float(x):
    v = alg._cfg_float({"inflation": x}, "inflation")
    assert v == float(np.float32(x)) == syn.float_config(x)


def test_rounding_is_visible_and_exact_values_pass_through():
    assert alg._cfg_float({"inflation": 1.1}, "inflation") == 1.100000023841858
    assert alg._cfg_float({"localization_radius": 6.5}, "localization_radius") == 6.5


def test_missing_config_key():
    with pytest.raises(KeyError):
        alg._cfg_float({}, "inflation")
    assert alg._cfg_float({}, "vertical_radius", 0.0) == 0.0
