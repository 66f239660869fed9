"""Writes the golden fixtures of tests/test_golden.py.

Each fixture is a short simulation drawn by the CPU oracle (oracle/clotho_oracle.cpp,
the restatement of the reference's per-generation step): the per-generation
tapes and the oracle's final state.  The GPU tests replay the tapes through
libclotho_gpu.so and must reproduce the rows, free list and allele tables bit
for bit.  Regenerate with:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

CASES = {
    # name: (oracle params, N or the list of per-generation sizes, generations)
    "neutral_wf": (dict(T=1, fitness=oracle.FIT_CONSTANT, mu=0.3, rho=0.5, p_neutral=1.0, seed=101), 64, 12),
    "qtl_two_traits": (dict(T=2, fitness=oracle.FIT_GAUSSIAN_VS, fit_param=4.0, mu=0.3, rho=2.0, p_neutral=0.3,
                            seed=202), 48, 10),
    "reference_gaussian_q1_off": (dict(T=1, fitness=oracle.FIT_GAUSSIAN, mu=0.4, rho=3.0, p_neutral=0.0, q1=False,
                                       seed=303), 40, 10),
    # small N, many generations: alleles fix, are cleared, recorded and their
    # slots reused (engine_batched_task.hpp:303-345)
    "drift_fixation": (dict(T=2, fitness=oracle.FIT_QUADRATIC, fit_param=2.0, mu=0.5, rho=0.5, p_neutral=0.5,
                            seed=404), 6, 60),
    # a size per generation (a growth model): growth, a fall below half (the parent individuals outnumber
    # the offspring rows), a one-individual bottleneck and regrowth
    "size_changes": (dict(T=2, fitness=oracle.FIT_GAUSSIAN_VS, fit_param=4.0, mu=0.6, rho=1.5, p_neutral=0.3,
                          seed=505), [60, 150, 20, 1, 3, 70, 200, 45], 8),
}


def make(name, params, N, G):
    sizes = list(N) if isinstance(N, list) else [N] * G
    assert len(sizes) == G
    orc = oracle.Oracle(threads=1, **params)
    orc.init(sizes[0])
    d = {"N": np.array([sizes[0]]), "Ncap": np.array([max(sizes)]), "G": np.array([G]),
         "T": np.array([params["T"]])}
    for k, v in params.items():
        d[f"param_{k}"] = np.array([v])
    for g in range(G):
        t = orc.step_record(sizes[g])
        d[f"g{g}_NM"] = np.array([t.N, t.M], np.int64)
        for f in ("pairs", "swap", "ev_off", "ev_pos", "mut_seq", "mut_pos", "mut_eff"):
            d[f"g{g}_{f}"] = getattr(t, f)
    info = orc.info()
    for k, v in info.items():
        d[f"info_{k}"] = np.array([v])
    d["rows"] = orc.rows()
    d["free"] = orc.free_list()
    pos, age, eff = orc.alleles()
    d["pos"], d["age"], d["eff"] = pos, age, eff
    fpos, fage, feff = orc.fixed()
    d["fixed_pos"], d["fixed_age"], d["fixed_eff"] = fpos, fage, feff
    d["phenotypes"] = orc.phenotypes()
    d["fitness"] = orc.fitness()
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **d)
    return info


if __name__ == "__main__":
    # python tests/golden/make_golden.py [name ...]  (all cases when none is named)
    for name, (params, N, G) in CASES.items():
        if len(sys.argv) > 1 and name not in sys.argv[1:]:
            continue
        info = make(name, params, N, G)
        print(name, info)
