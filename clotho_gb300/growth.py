"""Population growth: per-generation population sizes.

Restates the reference's growth plugins and their registry
(population_growth_toolkit.hpp:27-53, self-registered generators):

  linear      N' = (unsigned) (A * N + B)     linear_population_growth.cpp:23-25,
              A = 1, B = 0 by default         linear_population_growth_generator.cpp:17-22
  predefined  N' = sizes[g % len(sizes)]      predefined_population_growth.cpp:26-28,
              default sizes = [10000]         predefined_population_growth_generator.cpp:19-24

The engine calls the growth function with the current size and its
generation counter: once at set-up with (0, 0) for the initial size, then
before every generation g = 1, 2, ... with (N of the previous generation, g)
(engine_batched_task.hpp:143-170).  `schedule` produces that sequence, which
`Population.run_philox_schedule` / `Batch.run_schedule` replay on the device.
"""
from __future__ import annotations

from typing import Callable, Dict, List


class Growth:
    name = ""

    def __call__(self, N: int, generation: int) -> int:  # pragma: no cover - interface
        raise NotImplementedError

    def config(self) -> dict:  # pragma: no cover - interface
        raise NotImplementedError


class LinearGrowth(Growth):
    name = "linear"

    def __init__(self, A: float = 1.0, B: float = 0.0):
        self.A, self.B = float(A), float(B)

    def __call__(self, N: int, generation: int) -> int:
        v = self.A * N + self.B
        return int(v) if v > 0 else 0   # double -> unsigned conversion truncates toward zero

    def config(self) -> dict:
        return {"A": self.A, "B": self.B}


class PredefinedGrowth(Growth):
    name = "predefined"

    def __init__(self, sizes: List[int] | None = None):
        self.sizes = [int(s) for s in (sizes if sizes else [10000])]

    def __call__(self, N: int, generation: int) -> int:
        return self.sizes[generation % len(self.sizes)]

    def config(self) -> dict:
        return {"sizes": list(self.sizes)}


_REGISTRY: Dict[str, Callable[..., Growth]] = {}


def register(name: str, factory: Callable[..., Growth]):
    """Add a growth model under `name` (the toolkit's register_tool)."""
    _REGISTRY[name] = factory


def names():
    return sorted(_REGISTRY)


def from_config(config: dict) -> Growth:
    """`{"name": "linear", "A": 1.01, "B": 0}` or `{"name": "predefined", "sizes": [...]}`."""
    cfg = dict(config)
    name = cfg.pop("name")
    if name not in _REGISTRY:
        raise KeyError(f"unknown population growth model '{name}' (known: {', '.join(names())})")
    return _REGISTRY[name](**cfg)


register(LinearGrowth.name, LinearGrowth)
register(PredefinedGrowth.name, PredefinedGrowth)


def initial_size(growth: Growth) -> int:
    return growth(0, 0)


def schedule(growth: Growth, N: int, first_generation: int, G: int) -> List[int]:
    """Sizes of generations first_generation .. first_generation + G - 1,
    each computed from the previous one (N = the current size)."""
    out = []
    for g in range(first_generation, first_generation + G):
        N = growth(N, g)
        out.append(N)
    return out
