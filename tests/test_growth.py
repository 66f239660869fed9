"""Population growth models (CPU): the reference's linear and predefined
plugins and the order in which the engine applies them."""
import pytest

from clotho_gb300 import growth


def test_linear_truncates_like_the_reference():
    g = growth.LinearGrowth(1.05, 3.7)
    assert g(1000, 5) == int(1.05 * 1000 + 3.7)      # 1053.7 -> 1053
    assert growth.LinearGrowth()(1234, 9) == 1234    # A = 1, B = 0 by default
    assert growth.LinearGrowth(0.5, -100)(100, 1) == 0


def test_predefined_cycles_by_generation():
    g = growth.PredefinedGrowth([10, 20, 30])
    assert [g(0, k) for k in range(7)] == [10, 20, 30, 10, 20, 30, 10]
    assert growth.PredefinedGrowth()(0, 3) == 10000


def test_registry_and_schedule():
    assert growth.names() == ["linear", "predefined"]
    lin = growth.from_config({"name": "linear", "A": 2.0, "B": 1.0})
    assert growth.schedule(lin, 10, 1, 3) == [21, 43, 87]        # each from the previous size
    pre = growth.from_config({"name": "predefined", "sizes": [5, 6]})
    assert growth.initial_size(pre) == 5                           # set-up asks for generation 0
    assert growth.schedule(pre, 5, 1, 4) == [6, 5, 6, 5]
    with pytest.raises(KeyError):
        growth.from_config({"name": "exponential"})
