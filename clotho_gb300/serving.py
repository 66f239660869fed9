"""Continuous-batching serving loop.

Jobs (N, mu, rho, traits, generations, seed) arrive over time.  A job is
admitted when a population slot is free and its bitset footprint fits the
device budget; admitted jobs stay resident, and every step advances all of
them by one device-drawn generation in one launch per stage.  Jobs that reach
their generation count leave with their result (site-frequency spectrum,
mean fitness, segregating sites), which frees memory for the queue; their
column counts are taken inside the generation kernel during their last chunk
of generations, so the spectrum costs no extra pass over their rows.  Each
job's draws depend only on its own seed and generation counter, so its
result is the same alone and in the mix.

`run_plain` serves the same job list one job at a time (the plain engine).
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import Batch, make_desc, footprint_of, Population
from .config import neutral_capacity


@dataclass
class Job:
    id: int
    N: int
    mu: float
    rho: float
    T: int
    G: int
    seed: int
    arrival: float = 0.0
    fitness: str = "gaussian_vs"
    fit_param: float = 50.0
    p_neutral: float = 0.5
    # filled in
    admitted: float = math.nan
    done: float = math.nan
    result: dict = field(default_factory=dict)

    def max_alleles(self) -> int:
        return neutral_capacity(self.N, self.mu, self.G)

    def desc(self):
        return make_desc(self.N, self.max_alleles(), self.T, mu=self.mu, rho=self.rho, fitness=self.fitness,
                         fit_param=self.fit_param, p_neutral=self.p_neutral, seed=self.seed)

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def job_result(stats: dict, info: dict, sfs_len: int) -> dict:
    return {"sfs": stats.get("sfs", np.zeros(0)).tolist() if sfs_len else None,
            "mean_fitness": stats["mean_fitness"], "segregating": stats["segregating"],
            "generation": info["generation"] - 1, "device_error": info["device_error"]}


class Server:
    def __init__(self, budget_bytes: int, max_slots: int = 256, sfs_len: int = 64):
        self.batch = Batch()
        self.budget = budget_bytes
        self.max_slots = max_slots
        self.sfs_len = sfs_len
        self.queue: deque[Job] = deque()
        self.resident: list[tuple[Job, int]] = []   # (job, generations done)
        self.finished: list[Job] = []
        self.used = 0
        self.steps = 0
        self.counting: set[int] = set()   # resident indices whose population counts its columns
        self.peak_used = 0                 # bytes, and populations resident at once, at their highest
        self.peak_resident = 0

    def submit(self, job: Job):
        self.queue.append(job)

    def _admit(self, now: float):
        while self.queue and len(self.resident) < self.max_slots:
            job = self.queue[0]
            fp = footprint_of(job.desc())
            if self.used + fp > self.budget:
                if not self.resident and fp > self.budget:
                    raise RuntimeError(f"job {job.id} needs {fp} bytes, more than the budget")
                break
            self.queue.popleft()
            self.batch.add(job.desc(), job.N)
            self.used += fp
            job.admitted = now
            self.resident.append((job, 0))
            self.peak_used = max(self.peak_used, self.used)
            self.peak_resident = max(self.peak_resident, len(self.resident))

    def _retire(self, now: float):
        keep = []
        # remove from the highest index down so indices of the rest stay valid
        done_idx = [i for i, (job, g) in enumerate(self.resident) if g >= job.G]
        for i in sorted(done_idx, reverse=True):
            job, _ = self.resident[i]
            st = self.batch.stats(i, self.sfs_len)
            info = self.batch.info(i)
            job.result = job_result(st, info, self.sfs_len)
            job.done = now
            self.batch.remove(i)
            self.used -= footprint_of(job.desc())
            self.finished.append(job)
        # indices above a removed population shift down by one
        shifted = set()
        for c in self.counting:
            if c in done_idx:
                continue
            shifted.add(c - sum(1 for d in done_idx if d < c))
        self.counting = shifted
        for i, (job, g) in enumerate(self.resident):
            if i not in done_idx:
                keep.append((job, g))
        self.resident = keep

    def step(self, clock):
        self._admit(clock())
        if not self.resident:
            return False
        # advance every resident job; jobs with fewer generations left than the
        # chunk length retire inside it
        left = min(job.G - g for job, g in self.resident)
        k = max(1, min(left, 8))
        # jobs that finish in this chunk count their columns inside its generations, so their SFS is
        # read at retirement without another pass over the rows
        for i, (job, g) in enumerate(self.resident):
            if job.G - g <= k and i not in self.counting:
                self.batch.count_columns(i, True)
                self.counting.add(i)
        self.batch.run(k)
        self.batch.sync()
        self.resident = [(job, g + k) for job, g in self.resident]
        self.steps += k
        self._retire(clock())
        return True

    def run_open_loop(self, jobs: list[Job]) -> dict:
        jobs = sorted(jobs, key=lambda j: j.arrival)
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0  # noqa: E731
        pending = deque(jobs)
        while pending or self.queue or self.resident:
            now = clock()
            while pending and pending[0].arrival <= now:
                self.submit(pending.popleft())
            if not self.step(clock):
                if pending:
                    time.sleep(max(0.0, min(0.01, pending[0].arrival - clock())))
        return summarize(self.finished, clock())


def run_plain(jobs: list[Job], sfs_len: int = 64) -> dict:
    """The plain engine, one job at a time in arrival order."""
    jobs = sorted(jobs, key=lambda j: j.arrival)
    t0 = time.perf_counter()
    clock = lambda: time.perf_counter() - t0  # noqa: E731
    done = []
    for job in jobs:
        while clock() < job.arrival:
            time.sleep(min(0.01, job.arrival - clock()))
        d = job.desc()
        pop = Population(job.N, job.max_alleles(), job.T, mu=job.mu, rho=job.rho, fitness=job.fitness,
                         fit_param=job.fit_param, p_neutral=job.p_neutral, seed=job.seed,
                         max_events=d.max_events, max_mutations=d.max_mutations, max_fixed=d.max_fixed)
        pop.init(job.N)
        job.admitted = clock()
        pop.run_philox(job.N, job.G)
        pop.sync()
        st = pop.stats(sfs_len)
        info = pop.info()
        job.result = job_result(st, info, sfs_len)
        job.done = clock()
        pop.close()
        done.append(job)
    return summarize(done, clock())


def summarize(done: list[Job], makespan: float) -> dict:
    lat = np.array([j.latency for j in done]) if done else np.zeros(1)
    return {"jobs": len(done), "makespan_s": makespan, "jobs_per_s": len(done) / makespan if makespan else 0.0,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "errors": int(sum(1 for j in done if j.result.get("device_error")))}


def synthetic_jobs(n: int, rate: float, seed: int = 7, N_range=(1_000, 20_000), G_range=(50, 200),
                   mu_range=(1e-3, 1e-2), rho_range=(0.1, 5.0), traits=(1, 4)) -> list[Job]:
    """Poisson arrivals at `rate` jobs/s; N log-uniform, G / mu / rho uniform."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    jobs = []
    for i in range(n):
        N = int(np.exp(rng.uniform(np.log(N_range[0]), np.log(N_range[1]))))
        jobs.append(Job(id=i, N=N, mu=float(rng.uniform(*mu_range)), rho=float(rng.uniform(*rho_range)),
                        T=int(rng.integers(traits[0], traits[1] + 1)), G=int(rng.integers(G_range[0], G_range[1] + 1)),
                        seed=int(rng.integers(1, 2 ** 62)), arrival=float(t[i])))
    return jobs
