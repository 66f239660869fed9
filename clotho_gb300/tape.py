"""Event tape: the per-generation draws of a Clotho simulation.

The reference draws, per generation and in this order
(examples/QTLSim/engine_batched_task.hpp:175-202): the mutation count M
(mutation_allocator.hpp:41-47); N mate pairs (general_fitness_selection_generator.hpp:104-113);
for each of the 2N gametes E ~ Poisson(rho) breakpoints and their positions
(batch_crossover_mtwe.hpp:117-133); 2N strand-swap bits (:135-145); then per
mutation its target row, position and trait effects
(batch_mutation_task_population_space_row.hpp:76-88).  A tape holds exactly
those values, so any engine that consumes it reproduces the same genomes.

`neutral_tape` writes a tape for uniform parent choice (constant fitness)
with numpy, vectorised; it is the host-side producer used for end-to-end runs.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class GenTape:
    N: int
    M: int
    pairs: np.ndarray    # uint32 [2N]
    swap: np.ndarray     # uint8  [2N]
    ev_off: np.ndarray   # uint32 [2N+1]
    ev_pos: np.ndarray   # float64 [ev_off[-1]]
    mut_seq: np.ndarray  # uint32 [M]
    mut_pos: np.ndarray  # float64 [M]
    mut_eff: np.ndarray  # float32 [M*T]

    def contiguous(self) -> "GenTape":
        return GenTape(int(self.N), int(self.M),
                       np.ascontiguousarray(self.pairs, np.uint32), np.ascontiguousarray(self.swap, np.uint8),
                       np.ascontiguousarray(self.ev_off, np.uint32), np.ascontiguousarray(self.ev_pos, np.float64),
                       np.ascontiguousarray(self.mut_seq, np.uint32), np.ascontiguousarray(self.mut_pos, np.float64),
                       np.ascontiguousarray(self.mut_eff, np.float32))

    @property
    def nbytes(self) -> int:
        return int(sum(a.nbytes for a in (self.pairs, self.swap, self.ev_off, self.ev_pos, self.mut_seq,
                                          self.mut_pos, self.mut_eff)))


_FIELDS = ("pairs", "swap", "ev_off", "ev_pos", "mut_seq", "mut_pos", "mut_eff")


def save_tapes(path_or_file, tapes) -> None:
    """Store a list of GenTape in one .npz (generation i under key prefix g{i}_)."""
    d = {"count": np.array([len(tapes)], np.int64)}
    for i, t in enumerate(tapes):
        d[f"g{i}_NM"] = np.array([t.N, t.M], np.int64)
        for f in _FIELDS:
            d[f"g{i}_{f}"] = getattr(t, f)
    np.savez_compressed(path_or_file, **d)


def load_tapes(path_or_file):
    z = np.load(path_or_file)
    out = []
    for i in range(int(z["count"][0])):
        N, M = (int(v) for v in z[f"g{i}_NM"])
        out.append(GenTape(N, M, *(z[f"g{i}_{f}"] for f in _FIELDS)).contiguous())
    return out


def neutral_tape(rng: np.random.Generator, N: int, mu: float, rho: float, bias: float = 0.5, T: int = 1,
                 p_neutral: float = 1.0, eff_mean: float = 0.0, eff_sigma: float = 1.0,
                 parents: int | None = None) -> GenTape:
    """A generation of draws with uniform parents (constant fitness).

    parents: number of individuals in the parent population (default N)."""
    P = N if parents is None else parents
    S = 2 * N
    M = int(rng.poisson(mu * S))
    pairs = rng.integers(0, max(P, 1), size=S, dtype=np.uint32) if P > 0 else np.zeros(S, np.uint32)
    E = rng.poisson(rho, size=S).astype(np.uint32)
    ev_off = np.zeros(S + 1, np.uint32)
    np.cumsum(E, out=ev_off[1:])
    ev_pos = rng.random(int(ev_off[-1]))
    swap = (rng.random(S) < bias).astype(np.uint8)
    mut_seq = rng.integers(0, S, size=M, dtype=np.uint32)
    mut_pos = rng.random(M)
    eff = np.zeros((M, T), np.float32)
    if p_neutral < 1.0 and M:
        keep = rng.random((M, T)) >= p_neutral
        eff[keep] = (eff_mean + eff_sigma * rng.standard_normal(int(keep.sum()))).astype(np.float32)
    return GenTape(N, M, pairs, swap, ev_off, ev_pos, mut_seq, mut_pos, eff.reshape(-1))
