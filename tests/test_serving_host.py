"""The serving loop's host logic on CPU, against a stand-in for the device
batch: admission under the byte budget and the slot limit, retirement by
index from the highest down (every job gets its own population's result),
chunked stepping that never runs a job past its generation count, and the
error for a job larger than the whole budget; and the autotuner's search over
launch shapes and its cache.  The footprint of each job comes from the real
library (`clotho_footprint_for` needs no GPU)."""
import itertools
import math

import numpy as np
import pytest

import clotho_gb300 as cg
from clotho_gb300 import autotune, serving


class FakeBatch:
    """Resident populations as a list of [seed, generations run, generation at which column counting was
    switched on]; `run(k)` advances all of them, `stats`/`info` report the population at an index."""

    def __init__(self):
        self.pops = []
        self.runs = []
        self.peak = 0
        self.counted = []      # (seed, generations run, counting since) of every population read by stats

    def add(self, desc, N0=None):
        self.pops.append([desc.seed, 0, None])
        self.peak = max(self.peak, len(self.pops))
        return len(self.pops) - 1

    def count_columns(self, i, enable=True):
        assert enable and self.pops[i][2] is None
        self.pops[i][2] = self.pops[i][1]

    def remove(self, i):
        del self.pops[i]

    def run(self, k):
        self.runs.append((k, len(self.pops)))
        for p in self.pops:
            p[1] += k

    def sync(self):
        pass

    def stats(self, i, sfs_len=0):
        seed, gens, since = self.pops[i]
        self.counted.append((seed, gens, since))
        d = {"segregating": seed % 1000, "mean_fitness": float(seed), "fixed_now": 0, "heterozygosity": 0.0}
        if sfs_len:
            d["sfs"] = np.full(sfs_len, seed % 7, np.uint32)
        return d

    def info(self, i):
        return {"generation": self.pops[i][1] + 1, "device_error": 0}


@pytest.fixture
def fake(monkeypatch):
    made = []

    def make():
        b = FakeBatch()
        made.append(b)
        return b

    monkeypatch.setattr(serving, "Batch", make)
    return made


def _serve_all(srv, jobs):
    t = itertools.count()
    clock = lambda: float(next(t))  # noqa: E731
    for j in jobs:
        srv.submit(j)
    used_max = 0
    while srv.step(clock):
        used_max = max(used_max, srv.used)
        assert len(srv.resident) <= srv.max_slots
    return used_max


def test_every_job_runs_exactly_its_generations_and_gets_its_own_result(fake):
    jobs = serving.synthetic_jobs(40, rate=100.0, seed=3, N_range=(1_000, 5_000), G_range=(1, 30))
    srv = serving.Server(budget_bytes=1 << 40, max_slots=7, sfs_len=4)
    _serve_all(srv, jobs)
    b = fake[0]
    assert b.peak == 7 and not b.pops and not srv.queue and srv.used == 0
    assert sorted(j.id for j in srv.finished) == list(range(40))
    for j in srv.finished:
        assert j.result["generation"] == j.G, (j.id, j.G, j.result)
        assert j.result["mean_fitness"] == float(j.seed)
        assert j.result["sfs"] == [j.seed % 7] * 4
        assert j.admitted <= j.done
    assert all(1 <= k <= 8 for k, _ in b.runs)
    # every job counted its columns during its last chunk of generations only (the chunk is at most 8)
    by_seed = {j.seed: j for j in srv.finished}
    assert len(b.counted) == 40
    for seed, gens, since in b.counted:
        assert since is not None and by_seed[seed].G - 8 <= since < gens == by_seed[seed].G


def test_admission_keeps_the_budget(fake):
    jobs = serving.synthetic_jobs(30, rate=100.0, seed=5, N_range=(1_000, 20_000), G_range=(5, 20))
    fps = [cg.footprint_of(j.desc()) for j in jobs]
    budget = 3 * max(fps)
    srv = serving.Server(budget_bytes=budget, max_slots=64)
    used_max = _serve_all(srv, jobs)
    assert 0 < used_max <= budget
    assert len(srv.finished) == 30
    # jobs are admitted in arrival order (the queue is first in, first out)
    order = sorted(srv.finished, key=lambda j: (j.admitted, j.id))
    assert [j.id for j in order] == sorted(j.id for j in jobs)


def test_a_job_larger_than_the_budget_is_refused(fake):
    job = serving.synthetic_jobs(1, rate=1.0, seed=9)[0]
    srv = serving.Server(budget_bytes=cg.footprint_of(job.desc()) - 1)
    srv.submit(job)
    with pytest.raises(RuntimeError, match="more than the budget"):
        srv.step(lambda: 0.0)


def test_summary_percentiles():
    jobs = serving.synthetic_jobs(5, rate=1.0, seed=2)
    for i, j in enumerate(jobs):
        j.arrival, j.done, j.result = 0.0, float(i + 1), {"device_error": 1 if i == 4 else 0}
    s = serving.summarize(jobs, 5.0)
    assert s["jobs"] == 5 and s["jobs_per_s"] == 1.0 and s["p50_s"] == 3.0 and s["errors"] == 1


class TimedBatch:
    """Stand-in with a step cost (ms) per launch-shape configuration, for the autotuner."""

    def __init__(self, cost, N=(1000, 2000), A=4096):
        self.cost, self.N = cost, list(N)
        self.descs = [cg.make_desc(n, A) for n in N]
        self.cfg, self.steps, self.ms, self.trials = None, 0, 0.0, []

    def set_tuning(self, rows_per_item=0, narrow_build=1, row_blocks_per_sm=0):
        self.cfg = {"rows_per_item": rows_per_item, "narrow_build": narrow_build,
                    "row_blocks_per_sm": row_blocks_per_sm}
        self.trials.append(dict(self.cfg))

    def step(self):
        self.steps += 1
        self.ms += self.cost(self.cfg)

    def sync(self):
        pass

    def timer_begin(self):
        self.ms = 0.0

    def timer_end(self):
        return self.ms


def _cost(best):
    # separable cost with its minimum at `best`
    return lambda c: 1.0 + sum(abs(math.log2(c[k] + 1) - math.log2(best[k] + 1)) for k in best)


def test_autotuner_finds_the_fastest_shapes_and_caches_them(tmp_path):
    best = {"rows_per_item": 256, "narrow_build": 0, "row_blocks_per_sm": 8}
    b = TimedBatch(_cost(best))
    path = str(tmp_path / "sub" / "tune.json")
    assert autotune.tune(b, gens_per_trial=2, cache_path=path) == best and b.cfg == best
    n_trials = sum(len(v) for v in autotune.CANDIDATES.values())
    assert b.steps == 3 * n_trials                    # a warm-up and two timed steps per candidate
    b2 = TimedBatch(lambda c: 1.0)                     # a cache hit runs nothing
    assert autotune.tune(b2, cache_path=path) == best and b2.cfg == best and b2.steps == 0
    # another bucket (wider rows): the narrow build cannot run there, so that knob is not searched
    best3 = {"rows_per_item": 64, "narrow_build": 1, "row_blocks_per_sm": 24}
    b3 = TimedBatch(_cost(best3), A=1 << 20)
    assert autotune.bucket(b3) != autotune.bucket(b)
    got = autotune.tune(b3, cache_path=path)
    assert got == best3
    assert all(t["narrow_build"] == 1 for t in b3.trials)
    assert b3.steps == 3 * (n_trials - len(autotune.CANDIDATES["narrow_build"]))
