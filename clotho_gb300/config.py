"""QTLSim configuration files read into this engine's parameters.

QTLSim reads a JSON configuration (a Boost property tree: numbers may be
written as strings) from its `configuration` block, or from the root when that
block is absent (examples/QTLSim/qtlsim_main.cpp:111-113).  The keys and the
defaults each parameter object applies:

  generations.size                 10000   examples/generation_parameter.cpp:17-33
  population_growth.{name,params}  none    src/clotho/genetics/population_growth_toolkit.cpp:36-58
  mutation.mu                      1e-4    mutation/mutation_rate_parameter.hpp:24-39
  recombination.rho                1e-4    recombination/recombination_rate_parameter.hpp:24-39
  recombination.sequence_bias.p    0.5     recombination/sequence_bias_parameter.hpp:23-42
  traits.N                         1       phenotype_evaluator/trait_count_parameter.hpp:23-38
  traits.mean, traits.sigma        0, 1    generators/weight_parameter.hpp:38-41, random/normal_distribution_parameter.hpp:23-41
  neutral.p                        0.5     generators/neutral_parameter.hpp:35-50
  fitness.name                     ""      src/clotho/fitness/fitness_toolkit.cpp:50-69 ("" = no metric: constant)
  fitness.params.scale             1.0     fitness/quadratic_fitness_parameter.hpp:26-43 (the quadratic metric)
  random_number.seed               0       random/seed_parameter.hpp:25-46

Without a growth model the reference starts from zero individuals and keeps
the previous size every generation (engine_batched_task.hpp:143-170); with one,
the initial size is growth(0, 0).  The allele capacity has no key (the
reference grows its allele space as needed); `RunConfig.max_alleles` estimates
one from the neutral transient unless it is given.
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass, field
from typing import List, Optional

from . import growth as _growth

FITNESS_NAMES = {"": "constant", "constant": "constant", "gaussian": "gaussian", "quadratic": "quadratic"}


def neutral_capacity(N: int, mu: float, G: int) -> int:
    """Allele slots for a run of G generations at N individuals: about 1.5x the neutral transient's
    segregating sites, 2 N mu (1 + 2 ln G), at least 2,048 and at most 2^22."""
    est = 2.0 * N * mu * (1.0 + 2.0 * math.log(max(G, 2)))
    return int(min(1 << 22, max(2048, 1.5 * est + 1024)))


def _block(cfg: dict, key: str) -> dict:
    v = cfg.get(key, {})
    return v if isinstance(v, dict) else {}


@dataclass
class RunConfig:
    generations: int = 10000
    growth: Optional[_growth.Growth] = None
    mu: float = 1e-4
    rho: float = 1e-4
    bias: float = 0.5
    traits: int = 1
    eff_mean: float = 0.0
    eff_sigma: float = 1.0
    p_neutral: float = 0.5
    fitness: str = "constant"
    fit_param: float = 1.0
    seed: int = 0
    extra: dict = field(default_factory=dict)   # keys this engine does not use (threads, logging, ...)

    @property
    def N0(self) -> int:
        return _growth.initial_size(self.growth) if self.growth else 0

    def sizes(self) -> List[int]:
        """Individuals of generations 1 .. generations (the growth model's calls, in the engine's order)."""
        if not self.growth:
            return [self.N0] * self.generations
        return _growth.schedule(self.growth, self.N0, 1, self.generations)

    def max_individuals(self) -> int:
        return max([self.N0] + self.sizes()) if self.generations else self.N0

    def max_alleles(self) -> int:
        """The neutral capacity at the largest size."""
        return neutral_capacity(self.max_individuals(), self.mu, self.generations)

    def desc(self, max_alleles: int | None = None, **caps):
        from . import make_desc
        return make_desc(max(1, self.max_individuals()), max_alleles or self.max_alleles(), self.traits, mu=self.mu,
                         rho=self.rho, bias=self.bias, p_neutral=self.p_neutral, eff_mean=self.eff_mean,
                         eff_sigma=self.eff_sigma, fitness=self.fitness, fit_param=self.fit_param,
                         seed=self.seed, **caps)

    def population(self, max_alleles: int | None = None):
        """A device population with this configuration's parameters, initialised to the initial size."""
        from . import Population
        d = self.desc(max_alleles)
        pop = Population(d.max_individuals, d.max_alleles, self.traits, mu=self.mu, rho=self.rho, bias=self.bias,
                         p_neutral=self.p_neutral, eff_mean=self.eff_mean, eff_sigma=self.eff_sigma,
                         fitness=self.fitness, fit_param=self.fit_param, seed=self.seed,
                         max_events=d.max_events, max_mutations=d.max_mutations, max_fixed=d.max_fixed)
        pop.init(self.N0)
        return pop


def from_reference(config) -> RunConfig:
    """A QTLSim configuration (a dict, a JSON string or a path to a JSON file) as a RunConfig."""
    if isinstance(config, str):
        if config.lstrip().startswith("{"):
            config = json.loads(config)
        else:
            with open(config) as f:
                config = json.load(f)
    c = _block(config, "configuration") or config
    rc = RunConfig()
    rc.generations = int(float(_block(c, "generations").get("size", rc.generations)))
    g = _block(c, "population_growth")
    name = str(g.get("name", "") or "")
    if name:
        params = g.get("params", {})
        rc.growth = _growth.from_config(dict({"name": name}, **(params if isinstance(params, dict) else {})))
    rc.mu = float(_block(c, "mutation").get("mu", rc.mu))
    rec = _block(c, "recombination")
    rc.rho = float(rec.get("rho", rc.rho))
    rc.bias = float(_block(rec, "sequence_bias").get("p", rc.bias))
    tr = _block(c, "traits")
    rc.traits = int(float(tr.get("N", rc.traits)))
    rc.eff_mean = float(tr.get("mean", rc.eff_mean))
    rc.eff_sigma = float(tr.get("sigma", rc.eff_sigma))
    rc.p_neutral = float(_block(c, "neutral").get("p", rc.p_neutral))
    fit = _block(c, "fitness")
    fname = str(fit.get("name", "") or "")
    if fname not in FITNESS_NAMES:
        raise KeyError(f"unknown fitness metric '{fname}' (known: {', '.join(n for n in FITNESS_NAMES if n)})")
    rc.fitness = FITNESS_NAMES[fname]
    rc.fit_param = float(_block(fit, "params").get("scale", rc.fit_param)) if rc.fitness == "quadratic" else 1.0
    rc.seed = int(float(_block(c, "random_number").get("seed", rc.seed)))
    used = {"generations", "population_growth", "mutation", "recombination", "traits", "neutral", "fitness",
            "random_number"}
    rc.extra = {k: v for k, v in c.items() if k not in used}
    if not 1 <= rc.traits <= 4:
        raise ValueError(f"traits.N = {rc.traits}: this engine carries 1 to 4 traits")
    return rc
