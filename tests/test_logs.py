"""Reference-keyed log entries (CPU): margin_details::recordResults
(data_spaces/analysis/allele_frequency/margin_details.hpp:50-98) and the
performance / memory keys of Engine::getPerformanceResults."""
import numpy as np

from clotho_gb300 import logs


def test_allele_frequency_entry_from_margins():
    col = np.array([0, 3, 4, 1, 4, 2], np.uint32)   # 6 slots, 4 sequences
    row = np.array([3, 2, 5, 4], np.uint32)
    e = logs.allele_frequency(col, row, 4)
    assert e["distribution"] == [0, 3, 4, 1, 4, 2]
    assert e["frequency_distribution"] == [1, 1, 1, 1, 2]
    s = e["stats"]["sequences_per_allele"]
    assert (s["min"], s["max"], s["total"]) == (0, 4, 6)
    assert s["mean"] == 14 / 6
    assert abs(s["variance"] - np.var(col.astype(float))) < 1e-12   # divided by the count
    assert s["median"] == 2.5
    r = e["stats"]["alleles_per_sequence"]
    assert (r["min"], r["max"], r["mean"], r["total"]) == (2, 5, 3.5, 4)


def test_empty_population_entry():
    e = logs.allele_frequency(np.zeros(0, np.uint32), np.zeros(0, np.uint32), 0)
    assert e["distribution"] == [] and e["frequency_distribution"] == [0]
    assert e["stats"]["sequences_per_allele"]["total"] == 0


def test_performance_keys():
    p = logs.performance(1.5, [1.0, 2.0], [3, 4], [10, 11], [0, 1], {"crossover": [0.5, 0.6]})
    assert p["performance"]["runtime"] == 1.5 and p["performance"]["simulate"] == [1.0, 2.0]
    assert p["performance"]["crossover"] == [0.5, 0.6]
    assert p["memory"] == {"free_count": [3, 4], "variable_count": [10, 11], "fixed_count": [0, 1]}
