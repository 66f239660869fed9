"""QTLSim configuration files read into the engine's parameters (no GPU: the
descriptor is built on the host)."""
import ctypes
import json

import pytest

from clotho_gb300 import capi, config, growth

FULL = {"configuration": {
    "generations": {"size": "50"},
    "population_growth": {"name": "linear", "params": {"A": "1.1", "B": "300"}},
    "mutation": {"mu": "0.01"},
    "recombination": {"rho": "0.5", "sequence_bias": {"p": "0.3"}},
    "traits": {"N": "2", "mean": "0.1", "sigma": "2"},
    "neutral": {"p": "0.2"},
    "fitness": {"name": "quadratic", "params": {"scale": "3"}},
    "random_number": {"seed": "42"},
    "multithreading": {"T": "4"},
}}


def test_defaults_are_the_reference_parameter_defaults():
    rc = config.from_reference({})
    assert (rc.generations, rc.mu, rc.rho, rc.bias, rc.traits) == (10000, 1e-4, 1e-4, 0.5, 1)
    assert (rc.eff_mean, rc.eff_sigma, rc.p_neutral, rc.fitness, rc.seed) == (0.0, 1.0, 0.5, "constant", 0)
    assert rc.growth is None and rc.N0 == 0           # no growth model: the reference starts empty


def test_a_full_configuration_with_string_values():
    for cfg in (FULL, FULL["configuration"], json.dumps(FULL)):   # with or without the block, or as text
        rc = config.from_reference(cfg)
        assert rc.generations == 50 and rc.mu == 0.01 and rc.rho == 0.5 and rc.bias == 0.3
        assert rc.traits == 2 and rc.eff_mean == 0.1 and rc.eff_sigma == 2.0 and rc.p_neutral == 0.2
        assert rc.fitness == "quadratic" and rc.fit_param == 3.0 and rc.seed == 42
        assert isinstance(rc.growth, growth.LinearGrowth) and rc.N0 == 300
        assert rc.extra == {"multithreading": {"T": "4"}}
    sizes = rc.sizes()
    assert len(sizes) == 50 and sizes[0] == int(1.1 * 300 + 300) and sizes == growth.schedule(rc.growth, 300, 1, 50)
    assert rc.max_individuals() == max(sizes)


def test_predefined_growth_and_the_descriptor(tmp_path):
    cfg = {"population_growth": {"name": "predefined", "params": {"sizes": ["100", "40", "250"]}},
           "generations": {"size": 7}, "fitness": {"name": "gaussian"}, "traits": {"N": 3}}
    rc = config.from_reference(cfg)
    assert rc.N0 == 100 and rc.sizes() == [40, 250, 100, 40, 250, 100, 40]
    d = rc.desc()
    assert d.max_individuals == 250 and d.traits == 3 and d.max_alleles >= 2048
    assert d.fitness == 1 and d.fit_param == 1.0                     # the reference gaussian metric
    path = tmp_path / "qtlsim.json"
    path.write_text(json.dumps(cfg))
    assert config.from_reference(str(path)).sizes() == rc.sizes()   # read from a file


def test_unknown_metric_and_trait_counts_are_refused():
    with pytest.raises(KeyError, match="unknown fitness metric"):
        config.from_reference({"fitness": {"name": "random"}})
    with pytest.raises(KeyError, match="unknown population growth model"):
        config.from_reference({"population_growth": {"name": "logistic"}})
    with pytest.raises(ValueError, match="1 to 4 traits"):
        config.from_reference({"traits": {"N": 5}})


def test_footprint_of_the_configured_population_is_known_without_a_gpu():
    rc = config.from_reference(FULL)
    b = capi.load().clotho_footprint_for(ctypes.byref(rc.desc()))
    assert b > 2 * 2 * rc.max_individuals() * 8
