"""Autotuner for the launch shapes of a batched step.

Three knobs (clotho_set_tuning):
  rows_per_item      rows per scheduling item of the generation kernel: small
                     populations want small items (enough items to fill 152
                     SMs), large ones large items (fewer scheduling round trips);
  narrow_build       whether the generation kernel's narrow build (copy rows by
                     direct loads, every breakpoint's table words loaded at once)
                     may run when every row is at most 128 words;
  row_blocks_per_sm  blocks per SM of the per-individual kernels (parent
                     sampling, phenotype and fitness).
No knob changes a result (every kernel is deterministic in every shape), so the
tuning runs on the live batch: a coordinate search times a few generations per
candidate, one knob at a time with the others at their best so far, and keeps
the fastest.  Choices are cached per bucket of (population count, total rows,
widest allele capacity, trait mix)."""
from __future__ import annotations

import json
import math
import os

CANDIDATES = {
    "rows_per_item": (64, 128, 256, 512, 1024),
    "narrow_build": (1, 0),
    "row_blocks_per_sm": (16, 8, 4, 24),
}
DEFAULT = {"rows_per_item": 512, "narrow_build": 1, "row_blocks_per_sm": 16}
NARROW_MAX_ALLELES = 8192   # rows of at most 128 words: the narrow build can run


def bucket(batch) -> str:
    rows = sum(2 * n for n in batch.N)
    width = max((d.max_alleles for d in batch.descs), default=0)
    traits = sorted({d.traits for d in batch.descs})
    return (f"p{min(len(batch.N), 256).bit_length()}_r{int(math.log2(max(rows, 1)))}"
            f"_a{int(math.log2(max(width, 1)))}_t{''.join(str(t) for t in traits)}")


def knobs_for(batch) -> dict:
    """The knobs that can change anything on this batch (the narrow build needs every row <= 128 words)."""
    width = max((d.max_alleles for d in batch.descs), default=0)
    return {k: v for k, v in CANDIDATES.items() if k != "narrow_build" or width <= NARROW_MAX_ALLELES}


def _time(batch, cfg: dict, gens: int) -> float:
    batch.set_tuning(**cfg)
    batch.step()            # warm-up (and the graph capture for these shapes)
    batch.sync()
    batch.timer_begin()
    for _ in range(gens):
        batch.step()
    return batch.timer_end()


def tune(batch, gens_per_trial: int = 2, cache_path: str | None = None) -> dict:
    cache = {}
    if cache_path and os.path.exists(cache_path):
        with open(cache_path) as f:
            cache = json.load(f)
    key = bucket(batch)
    if key in cache and isinstance(cache[key], dict):
        cfg = dict(DEFAULT, **cache[key])
        batch.set_tuning(**cfg)
        return cfg
    cfg = dict(DEFAULT)
    for knob, cands in knobs_for(batch).items():
        best, best_ms = cfg[knob], float("inf")
        for v in cands:
            ms = _time(batch, dict(cfg, **{knob: v}), gens_per_trial)
            if ms < best_ms:
                best, best_ms = v, ms
        cfg[knob] = best
    batch.set_tuning(**cfg)
    cache[key] = cfg
    if cache_path:
        os.makedirs(os.path.dirname(os.path.abspath(cache_path)), exist_ok=True)
        with open(cache_path, "w") as f:
            json.dump(cache, f, indent=1)
    return cfg
