"""Synthetic workloads with the shapes of the reference's published configurations.

No public dataset is involved: every input is seeded synthetic data.

* neutral_wf      N=1e4 diploid, mu=0.01, rho=0.01, uniform parents, 1,000 generations.
* qtl_selection   N=1e5, mu=0.1, rho=1.0, one trait, effects N(0,1), exp(-z^2/2), 2,000 generations.
* large_n         N=1e6, 4 traits, effects N(0,I), 65,536 allele slots (W=1,024 words),
                  device Philox draws.  As literally stated (mu=1.0 per sequence) it asks
                  for 2e6 new alleles per generation, more than the 65,536 slots; it is
                  measured from a pre-seeded steady load (neutral 1/i spectrum over the
                  slots) with mu=1e-3, rho=5.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    N: int
    mu: float
    rho: float
    T: int
    fitness: str
    fit_param: float
    p_neutral: float
    generations: int
    max_alleles: int
    seeded_alleles: int = 0          # pre-seeded slots (0 = empty start, Engine::init)
    bias: float = 0.5
    extra: dict = field(default_factory=dict)


NEUTRAL_WF = Workload("neutral_wf N=1e4 mu=0.01 rho=0.01", 10_000, 0.01, 0.01, 1, "constant", 1.0, 1.0, 1000,
                      8192)
QTL_SELECTION = Workload("qtl_selection N=1e5 mu=0.1 rho=1 T=1 exp(-z^2/2)", 100_000, 0.1, 1.0, 1, "gaussian_vs",
                         1.0, 0.0, 2000, 1 << 19)
LARGE_N = Workload("large_n N=1e6 T=4 A=65536 (W=1024) rho=5 mu=1e-3 pre-seeded", 1_000_000, 1e-3, 5.0, 4,
                   "gaussian", 1.0, 0.0, 500, 65_536, seeded_alleles=58_000)


def neutral_spectrum_thresholds(rng: np.random.Generator, S: int, A: int) -> np.ndarray:
    """Per-slot carrier probabilities drawn from the neutral spectrum P(i) ~ 1/i,
    i in [1, S-1] carriers out of S sequences, returned as uint32 thresholds
    (bit set iff hash < thr)."""
    i = np.arange(1, S, dtype=np.float64)
    cdf = np.cumsum(1.0 / i)
    cdf /= cdf[-1]
    k = np.searchsorted(cdf, rng.random(A), side="right") + 1
    k = np.minimum(k, S - 1)
    return np.minimum(np.floor(k / S * 2.0 ** 32), 2.0 ** 32 - 1).astype(np.uint32)


def seeded_start(w: Workload, seed: int = 20261203, N: int | None = None):
    """Host arrays for clotho_seed_population / orc_seed_population:
    positions U[0,1), effects N(0,1) FP32 (p_neutral applied), thresholds."""
    N = w.N if N is None else N
    rng = np.random.default_rng(seed)
    A = w.seeded_alleles
    pos = rng.random(A)
    eff = rng.standard_normal((A, w.T)).astype(np.float32)
    if w.p_neutral > 0:
        eff[rng.random((A, w.T)) < w.p_neutral] = 0.0
    thr = neutral_spectrum_thresholds(rng, 2 * N, A)
    return pos, eff.reshape(-1), thr
