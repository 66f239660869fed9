"""The serving loop's host logic on CPU, against a stand-in for the device
batch: admission under the byte budget and the slot limit, retirement by
index from the highest down (every job gets its own population's result),
chunked stepping that never runs a job past its generation count, and the
error for a job larger than the whole budget; and the autotuner's choice of
rows per item and its cache.  The footprint of each job comes from the real
library (`clotho_footprint_for` needs no GPU)."""
import itertools

import numpy as np
import pytest

import clotho_gb300 as cg
from clotho_gb300 import autotune, serving


class FakeBatch:
    """Resident populations as a list of [seed, generations run]; `run(k)`
    advances all of them, `stats`/`info` report the population at an index."""

    def __init__(self):
        self.pops = []
        self.runs = []
        self.peak = 0

    def add(self, desc, N0=None):
        self.pops.append([desc.seed, 0])
        self.peak = max(self.peak, len(self.pops))
        return len(self.pops) - 1

    def remove(self, i):
        del self.pops[i]

    def run(self, k):
        self.runs.append((k, len(self.pops)))
        for p in self.pops:
            p[1] += k

    def sync(self):
        pass

    def stats(self, i, sfs_len=0):
        seed, gens = self.pops[i]
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
    """Stand-in with a per-grain step cost (ms), for the autotuner."""

    def __init__(self, cost, N=(1000, 2000), A=4096):
        self.cost, self.N = cost, list(N)
        self.descs = [cg.make_desc(n, A) for n in N]
        self.rpi, self.steps, self.ms = None, 0, 0.0

    def set_rows_per_item(self, r):
        self.rpi = r

    def step(self):
        self.steps += 1
        self.ms += self.cost[self.rpi]

    def sync(self):
        pass

    def timer_begin(self):
        self.ms = 0.0

    def timer_end(self):
        return self.ms


def test_autotuner_keeps_the_fastest_grain_and_caches_it(tmp_path):
    cost = {64: 5.0, 128: 3.0, 256: 1.5, 512: 2.0, 1024: 4.0}
    b = TimedBatch(cost)
    path = str(tmp_path / "sub" / "tune.json")
    assert autotune.tune(b, gens_per_trial=2, cache_path=path) == 256 and b.rpi == 256
    assert b.steps == 3 * len(autotune.CANDIDATES)
    b2 = TimedBatch({k: 1.0 for k in cost})  # a cache hit runs nothing
    assert autotune.tune(b2, cache_path=path) == 256 and b2.rpi == 256 and b2.steps == 0
    # another bucket (wider rows) is tuned afresh
    b3 = TimedBatch({64: 1.0, 128: 2.0, 256: 3.0, 512: 4.0, 1024: 5.0}, A=1 << 20)
    assert autotune.bucket(b3) != autotune.bucket(b)
    assert autotune.tune(b3, cache_path=path) == 64
