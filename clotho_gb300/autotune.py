"""Autotuner for the generation kernel's scheduling grain (rows per item).

Small populations want small items (enough items to fill 152 SMs); large ones
want large items (fewer scheduling round trips).  Results are independent of
the grain (the kernel is deterministic), so tuning runs on the live batch:
each candidate times a few generations and the fastest is kept, cached per
bucket of (population count, total rows, widest row)."""
from __future__ import annotations

import json
import math
import os

CANDIDATES = (64, 128, 256, 512, 1024)


def bucket(batch) -> str:
    rows = sum(2 * n for n in batch.N)
    width = max((d.max_alleles for d in batch.descs), default=0)
    return f"p{min(len(batch.N), 256).bit_length()}_r{int(math.log2(max(rows, 1)))}_a{int(math.log2(max(width, 1)))}"


def tune(batch, gens_per_trial: int = 2, cache_path: str | None = None) -> int:
    cache = {}
    if cache_path and os.path.exists(cache_path):
        with open(cache_path) as f:
            cache = json.load(f)
    key = bucket(batch)
    if key in cache:
        batch.set_rows_per_item(int(cache[key]))
        return int(cache[key])
    best, best_ms = CANDIDATES[0], float("inf")
    for rpi in CANDIDATES:
        batch.set_rows_per_item(rpi)
        batch.step()            # warm-up (and the graph capture for this grain)
        batch.sync()
        batch.timer_begin()
        for _ in range(gens_per_trial):
            batch.step()
        ms = batch.timer_end()
        if ms < best_ms:
            best, best_ms = rpi, ms
    batch.set_rows_per_item(best)
    cache[key] = best
    if cache_path:
        os.makedirs(os.path.dirname(os.path.abspath(cache_path)), exist_ok=True)
        with open(cache_path, "w") as f:
            json.dump(cache, f, indent=1)
    return best
