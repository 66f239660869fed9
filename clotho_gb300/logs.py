"""Log entries with the reference's keys.

`allele_frequency` restates margin_details::recordResults
(data_spaces/analysis/allele_frequency/margin_details.hpp:50-98), the entry
population_analyzer writes for every sample (examples/QTLSim/qtlsim_main.cpp:
201-221): the column margins as `distribution`, the number of allele slots
carried by exactly k sequences as `frequency_distribution`, and min / max /
mean / median / variance / total of the column margins
(`sequences_per_allele`) and of the row margins (`alleles_per_sequence`).

Statistics follow Boost.Accumulators' definitions: `variance` is the
population variance (divided by the count).  `median` here is the exact
median; Boost's `tag::median` is the P-square estimate, so the two can differ
on skewed margins.

`performance` builds the `performance.*` and `memory.*` keys of
Engine::getPerformanceResults (examples/QTLSim/engine_batched_task.hpp:
233-242) and qtlsim_main.cpp:183-192 from per-generation records.
"""
from __future__ import annotations

import numpy as np


def _stats(v) -> dict:
    v = np.asarray(v, np.float64)
    if v.size == 0:
        return {"min": 0, "max": 0, "mean": 0.0, "median": 0.0, "variance": 0.0, "total": 0}
    return {"min": int(v.min()), "max": int(v.max()), "mean": float(v.mean()),
            "median": float(np.median(v)), "variance": float(v.var()), "total": int(v.size)}


def allele_frequency(col_counts, row_counts, sequences: int) -> dict:
    """The `allele_frequency` entry from the margins of the current rows.

    col_counts: sequences carrying each allele slot (length A).
    row_counts: alleles carried by each sequence (length 2N).
    sequences:  2N.  `frequency_distribution[k]` counts slots carried by
    exactly k sequences, k = 0..2N.
    """
    col = np.asarray(col_counts, np.int64)
    row = np.asarray(row_counts, np.int64)
    freq = np.bincount(col, minlength=sequences + 1) if col.size else np.zeros(sequences + 1, np.int64)
    return {
        "distribution": [int(x) for x in col],
        "frequency_distribution": [int(x) for x in freq],
        "stats": {"sequences_per_allele": _stats(col), "alleles_per_sequence": _stats(row)},
    }


def performance(runtime_s: float, simulate_ms, free_counts, variable_counts, fixed_counts,
                stage_ms: dict | None = None) -> dict:
    """`performance.*` and `memory.*` keys from per-generation records."""
    out = {"performance": {"runtime": float(runtime_s), "simulate": [float(x) for x in simulate_ms]},
           "memory": {"free_count": [int(x) for x in free_counts],
                      "variable_count": [int(x) for x in variable_counts],
                      "fixed_count": [int(x) for x in fixed_counts]}}
    for k, v in (stage_ms or {}).items():  # mutate / crossover / fixed / phenotypes
        out["performance"][k] = [float(x) for x in v]
    return out
