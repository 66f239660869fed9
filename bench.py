#!/usr/bin/env python3
"""bench.py -- sequence-generations/s of Clotho's per-generation hot path on GB300.

Workload: N=1e6 diploid (2e6 rows), 4 traits, 65,536 allele slots (W<=1,024
words per row), rho=5, mu=1e-3 per sequence, pre-seeded neutral 1/i load,
device Philox draws, reference `gaussian` fitness (sigma = sqrt(4 N mu)),
fitness-proportional parents from an FP64 prefix sum.  One step = one
generation (free space, selection, crossover, mutation, phenotype, fitness).

  value    device-resident throughput, K generations replayed from one CUDA graph.
  e2e      the same metric through the C-ABI tape call with host buffers: every
           step copies that generation's tape from pinned host memory and reads
           the step's status (mean fitness) back.
  roofline the fused generation kernel: algorithmic bytes 16*W_live*S per launch
           (each child row written once, each selected parent row read once)
           over its CUDA-event duration, against MEASURED_PEAKS.json hbm_gbs.
  cpu_baseline  the CPU oracle (restatement of the reference's path) on the
           host cores, on a bounded sample of the same workload.
  configs  the neutral (N=1e4, 1,000 generations) and QTL-with-selection
           (N=1e5, 2,000 generations) configurations as stated, on the GPU and
           the CPU restatement, with the FP32-vs-FP64 phenotype error.

--impl reference times that CPU restatement alone, on this arm's configuration
(N=1e6, all host threads), with the single-core rate beside it: the
reference's own engine needs Boost (every hot-path header includes it), which
this image lacks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sequence-generations/s at N=1e6 (HBM % peak)"
UNIT = "seq-gen/s"
FALLBACK_HBM_GBS = 6800.0
CPU_SAMPLE_N = 20_000     # single-core sample (individuals)
CPU_LEG_N = 100_000       # all-cores sample of the in-line CPU leg (individuals)
REF_N = None              # individuals of the reference arm (None: the workload's own N)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", type=int, default=None, help="override N (small runs / profiling)")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--profile-gens", type=int, default=4)
    p.add_argument("--kernel-only", action="store_true", help="seed + eager generations only (ncu runs)")
    p.add_argument("--batch-kernels", action="store_true",
                   help="the batched workload's 256 populations, warmup + steps eager generations only (ncu runs)")
    p.add_argument("--phase-clocks", action="store_true",
                   help="print the generation kernel's per-phase cycle breakdown (profiling build) and exit")
    p.add_argument("--no-batched", action="store_true", help="skip the batched and serving measurements")
    p.add_argument("--no-configs", action="store_true",
                   help="skip the neutral and QTL-with-selection configurations (GPU and CPU)")
    p.add_argument("--configs-only", action="store_true",
                   help="only the neutral and QTL-with-selection configurations")
    p.add_argument("--batched-only", action="store_true", help="only the batched and serving measurements")
    p.add_argument("--qtl-kernel", type=int, default=0, metavar="G",
                   help="the QTL-with-selection configuration from an empty start for G + warmup + steps eager "
                        "generations (ncu runs of the interval-classifier kernel)")
    p.add_argument("--c4-waves", action="store_true",
                   help="the batched configuration with mu U[0.01,0.05] through footprint-admitted waves (one-off)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max-reduce over replicas (gloo; the data path has no collective)."""

    def __init__(self, world):
        self.world = world
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if not self.dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic():
    path = os.path.join(ROOT, "profiles", "generation_kernel_traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        with open(self.path) as f:
            out = self.parse(f)
        os.unlink(self.path)
        return out

    @staticmethod
    def parse(lines):
        """Median SM clock, max SM clock and the throttle reasons seen Active in
        nvidia-smi's csv,noheader,nounits rows of FIELDS."""
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_population(cg, w, N, extra_fixed=1 << 20):
    return cg.Population(N, w.max_alleles, w.T, fitness=w.fitness, fit_param=w.fit_param, mu=w.mu, rho=w.rho,
                         bias=w.bias, p_neutral=w.p_neutral, seed=20261203, max_fixed=extra_fixed,
                         max_events=int(2 * N * w.rho * 1.05 + 4096), max_mutations=int(2 * N * w.mu * 1.5 + 4096))


def pinned_tape(cg, tape):
    """Copy a GenTape into one page-locked block; returns (tape view, keepalive)."""
    import numpy as np
    L = cg.capi.load()
    t = tape.contiguous()
    arrs = [t.pairs, t.swap, t.ev_off, t.ev_pos, t.mut_seq, t.mut_pos, t.mut_eff]
    offs, total = [], 0
    for a in arrs:
        total = (total + 63) & ~63
        offs.append(total)
        total += a.nbytes
    ptr = C.c_void_p()
    if L.clotho_host_alloc(max(total, 64), C.byref(ptr)) != 0:
        raise RuntimeError("clotho_host_alloc failed")
    buf = (C.c_char * max(total, 64)).from_address(ptr.value)
    views = []
    for a, o in zip(arrs, offs):
        v = np.frombuffer(buf, dtype=a.dtype, count=a.size, offset=o)
        v[...] = a
        views.append(v)
    out = cg.GenTape(t.N, t.M, *views)
    return out, ptr


def run_cpu_oracle(w, N, steps, warmup, threads):
    """The CPU restatement on the host cores: bounded sample of the workload
    (N individuals, same allele load and per-row width)."""
    import oracle
    from clotho_gb300.workloads import seeded_start
    fit = {"constant": oracle.FIT_CONSTANT, "gaussian": oracle.FIT_GAUSSIAN, "quadratic": oracle.FIT_QUADRATIC,
           "gaussian_vs": oracle.FIT_GAUSSIAN_VS}[w.fitness]
    orc = oracle.Oracle(T=w.T, fitness=fit, fit_param=w.fit_param, mu=w.mu, rho=w.rho, bias=w.bias,
                        p_neutral=w.p_neutral, q1=True, threads=threads, seed=7)
    pos, eff, thr = seeded_start(w, N=N)
    orc.seed_population(N, pos, eff, thr, 99)
    for _ in range(warmup):
        orc.step_record(N)
    t0 = time.perf_counter()
    stages = {}
    for _ in range(steps):
        orc.step_record(N)
        for k, v in orc.times().items():
            stages[k] = stages.get(k, 0.0) + v
    dt = time.perf_counter() - t0
    info = orc.info()
    orc.close()
    return 2.0 * N * steps / dt, dt, info, stages


def compare_batched(cg, serving, autotune, N_range, G, n=256, seed=11):
    """One batch of n populations against the same jobs one at a time, both arms timed alike: with set-up
    (context creation, init, generations, teardown) and steady state (generations only).  The tuner's
    choice is made on a separate batch of the same jobs (it is cached per bucket in use)."""
    jobs = serving.synthetic_jobs(n, rate=1e9, seed=seed, N_range=N_range, G_range=(G, G))
    descs = [j.desc() for j in jobs]
    t0 = time.perf_counter()
    bt = cg.Batch(descs)
    bt.init()
    tuned = autotune.tune(bt, gens_per_trial=2)
    bt.close()
    t_tune = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = cg.Batch(descs)
    b.init()
    b.set_tuning(**tuned)
    b.sync()
    t1 = time.perf_counter()
    b.run(G)
    b.sync()
    t2 = time.perf_counter()
    errs = sum(1 for i in range(len(jobs)) if b.info(i)["device_error"])
    footprint = b.footprint
    b.close()
    t3 = time.perf_counter()
    b_setup, b_steady = t3 - t0, t2 - t1
    p_setup = p_steady = 0.0
    for j in jobs:
        d = j.desc()
        t0 = time.perf_counter()
        pop = cg.Population(j.N, j.max_alleles(), j.T, mu=j.mu, rho=j.rho, fitness=j.fitness,
                            fit_param=j.fit_param, p_neutral=j.p_neutral, seed=j.seed, max_events=d.max_events,
                            max_mutations=d.max_mutations, max_fixed=d.max_fixed)
        pop.init(j.N)
        pop.sync()
        t1 = time.perf_counter()
        pop.run_philox(j.N, G)
        pop.sync()
        t2 = time.perf_counter()
        pop.close()
        t3 = time.perf_counter()
        p_setup += t3 - t0
        p_steady += t2 - t1
    return {
        "with_setup": {"jobs_per_s": n / b_setup, "plain_jobs_per_s": n / p_setup, "speedup": p_setup / b_setup,
                       "note": "batched: Batch creation, init, generations, teardown; plain: Population creation, "
                               "init, generations, teardown for every job"},
        "steady": {"jobs_per_s": n / b_steady, "plain_jobs_per_s": n / p_steady, "speedup": p_steady / b_steady,
                   "note": "generations only, in both arms"},
        "jobs_per_s": n / b_setup, "plain_jobs_per_s": n / p_setup, "speedup": p_setup / b_setup,
        "tuning": tuned, "autotune_s": t_tune, "device_errors": errs, "footprint_gb": footprint / 1e9}


def c4_waves(budget_gb: int = 200, G: int = 50):
    """The batched configuration's N, rho and trait ranges with mu at the low end of its stated range
    (U[0.01, 0.05]): ~390 GB of populations, more than the device holds, so they run through the serving
    loop's footprint admission, all arriving at once (waves: a population is admitted when its bitsets fit
    the budget, and leaves when it reaches G); against the same jobs one at a time."""
    import clotho_gb300 as cg
    from clotho_gb300 import serving
    jobs = serving.synthetic_jobs(256, rate=1e9, seed=11, N_range=(1_000, 200_000), G_range=(G, G),
                                  mu_range=(0.01, 0.05))
    for j in jobs:
        j.arrival = 0.0
    total = sum(cg.footprint_of(j.desc()) for j in jobs)
    big = sum(1 for j in jobs if j.max_alleles() > 65_536)
    pjobs = [serving.Job(**{k: getattr(j, k) for k in ("id", "N", "mu", "rho", "T", "G", "seed", "arrival")})
             for j in jobs]
    srv = serving.Server(budget_bytes=budget_gb << 30, max_slots=256)
    s_srv = srv.run_open_loop(jobs)
    s_plain = serving.run_plain(pjobs)
    same = sum(1 for j, p in zip(sorted(srv.finished, key=lambda x: x.id), pjobs)
               if j.result["sfs"] == p.result["sfs"] and j.result["mean_fitness"] == p.result["mean_fitness"])
    return {"c4_waves": {
        "workload": (f"256 populations, N log-U[1e3,2e5], mu U[0.01,0.05], rho U[0.1,5], T 1-4, G={G}: "
                     f"{total / 1e9:.0f} GB of populations ({big} above 65,536 allele slots), through a "
                     f"{budget_gb} GB admission budget"),
        "served": s_srv, "plain": s_plain, "speedup_jobs_per_s": s_srv["jobs_per_s"] / s_plain["jobs_per_s"],
        "peak_resident": srv.peak_resident, "peak_used_gb": srv.peak_used / 1e9, "identical_results": same}}


def batched_and_serving():
    """Batched populations and continuous-batching serving against the plain engine one job at a time, on
    synthetic job mixes shaped like the batched and serving configurations (named deviations in `workload`),
    with both arms timed alike."""
    import clotho_gb300 as cg
    from clotho_gb300 import serving, autotune

    batched = compare_batched(cg, serving, autotune, N_range=(1_000, 200_000), G=100)
    batched["workload"] = (
        f"256 populations, N log-U[1e3,2e5], mu U[1e-3,1e-2], rho U[0.1,5], T 1-4, G=100, all resident "
        f"({batched.pop('footprint_gb'):.0f} GB). Deviations from the batched configuration: mu (stated U[0.01,1.0]; "
        "at N=2e5 that is up to 6e6 allele slots, ~590 GB for one population) and G (stated 1,000; 100 keeps both "
        "arms within a minute). Large populations fill the GPU on their own, so batching gains little on them")
    small = compare_batched(cg, serving, autotune, N_range=(1_000, 20_000), G=100)
    small["workload"] = (f"256 populations, N log-U[1e3,2e4], mu U[1e-3,1e-2], rho U[0.1,5], T 1-4, G=100 "
                         f"({small.pop('footprint_gb'):.0f} GB): small populations, where one-at-a-time runs are "
                         "bound by launches and set-up")
    batched["small_populations"] = small
    batched["waves"] = c4_waves()["c4_waves"]

    # ---- serving: open-loop Poisson arrivals at 20 jobs/s, both arms on the same job list
    sjobs = serving.synthetic_jobs(200, rate=20.0, seed=21, N_range=(1_000, 10_000), G_range=(200, 2000))
    pjobs = [serving.Job(**{k: getattr(j, k) for k in ("id", "N", "mu", "rho", "T", "G", "seed", "arrival")})
             for j in sjobs]
    srv = serving.Server(budget_bytes=64 << 30, max_slots=256)
    s_srv = srv.run_open_loop(sjobs)
    s_plain = serving.run_plain(pjobs)      # busy from the first arrival on: its jobs/s is its capacity
    cjobs = [serving.Job(**{k: getattr(j, k) for k in ("id", "N", "mu", "rho", "T", "G", "seed")}, arrival=0.0)
             for j in sjobs]
    cap = serving.Server(budget_bytes=64 << 30, max_slots=256).run_open_loop(cjobs)
    same = sum(1 for j, p in zip(sorted(srv.finished, key=lambda x: x.id), pjobs)
               if j.result["sfs"] == p.result["sfs"] and j.result["mean_fitness"] == p.result["mean_fitness"])
    serve = {"workload": ("200 jobs arriving as a Poisson stream at 20 jobs/s (the serving configuration's rate), "
                          "G U[200,2000] (as stated), N log-U[1e3,1e4] (stated 1e3-5e5: one 5e5 job of 2,000 "
                          "generations takes ~15 s on the plain engine, the whole run a few hours), mu U[1e-3,1e-2] "
                          "(unstated), rho U[0.1,5], T 1-4; latency = completion - arrival"),
             "served": s_srv, "plain": s_plain, "speedup_jobs_per_s": s_srv["jobs_per_s"] / s_plain["jobs_per_s"],
             "served_capacity": {**cap, "note": "the same jobs all arriving at once: the served loop's capacity "
                                 "(at 20 jobs/s it is bound by the arrivals; the plain engine is saturated there)"},
             "capacity_speedup": cap["jobs_per_s"] / s_plain["jobs_per_s"],
             "identical_results": same}
    return batched, serve


def drop_in_rate(N, w, gens=3):
    """The C++ drop-in engine (clotho_gb300/cpp, EngineGB300 through the tape call) at this N: every generation's
    draws made on the host in the reference's order with a serial generator (std::mt19937_64: parents from the
    fitness, 2N breakpoint counts and their positions, swap bits, new alleles), then one tape call.  Starts from
    an empty population (its rows stay narrow), so the time is the host draws' plus a small device share."""
    from clotho_gb300 import builder
    try:
        out = subprocess.run([builder.DRIVER_PATH, str(N), str(gens), str(w.mu), str(w.rho), str(w.T), "0", "7"],
                             capture_output=True, text=True, timeout=600, check=True).stdout
        perf = json.loads(out.strip().splitlines()[-1])["performance"]["simulate"][1:]
    except Exception as e:  # the driver is a convenience measurement; the line stands without it
        return {"error": str(e)[:200]}
    s = statistics.mean(perf)
    return {"value": 2.0 * N / s, "unit": UNIT, "ms_per_step": 1e3 * s,
            "note": "C++ drop-in (tape mode): the reference's draws on the host with one serial generator, then "
                    "the tape call; the host draws bound it (generations after the first, whose uniform parents "
                    "are cheaper to draw)"}


def stated_configs(cg, threads):
    """The neutral (N=1e4, G=1,000) and QTL-with-selection (N=1e5, G=2,000) configurations as stated, from an
    empty start with device draws, in one graph-replayed call each; then the rate and the generation kernel's
    bandwidth at the final load, and the CPU restatement on the same final state (all host threads and one),
    with the FP32-carried phenotypes of the QTL run against the FP64 sums of its rows."""
    import numpy as np
    import oracle
    from clotho_gb300.workloads import NEUTRAL_WF, QTL_SELECTION
    fits = {"constant": oracle.FIT_CONSTANT, "gaussian_vs": oracle.FIT_GAUSSIAN_VS}
    peak, peak_kind = measured_peak()
    out = {}
    for key, w, cpu_gens in (("neutral_wf", NEUTRAL_WF, 1000), ("qtl_selection", QTL_SELECTION, 6)):
        pop = cg.Population(w.N, w.max_alleles, w.T, fitness=w.fitness, fit_param=w.fit_param, mu=w.mu, rho=w.rho,
                            bias=w.bias, p_neutral=w.p_neutral, seed=20261203, max_fixed=1 << 20)
        pop.init(w.N)
        pop.sync()
        pop.timer_begin()
        pop.run_philox(w.N, w.generations)
        ms = pop.timer_end()
        pop.sync()
        pop.check()
        whole = 2.0 * w.N * w.generations / (ms / 1e3)
        pop.timer_begin()
        pop.run_philox(w.N, 20)
        ms_f = pop.timer_end()
        pop.profile(True)
        for _ in range(4):
            pop.simulate_philox(w.N)
        kms, nl, rows_done, words_done = pop.kernel_time()
        pop.profile(False)
        pop.check()
        info = pop.info()
        kern_ms = kms / max(nl, 1)
        gbs = 16.0 * words_done / max(nl, 1) / (kern_ms / 1e3) / 1e9
        gpu = {"seq_gen_per_s": whole, "generations": w.generations, "s": ms / 1e3,
               "final": {"generation": info["generation"], "A": info["A"], "W": info["W"],
                         "seq_gen_per_s": 2.0 * w.N * 20 / (ms_f / 1e3), "ms_per_generation": ms_f / 20,
                         "kernel_ms": kern_ms, "achieved_gbs": gbs, "frac": gbs / peak,
                         "peak_kind": f"of {peak_kind}"}}
        rows = pop.rows()
        pos, _, eff = pop.alleles()
        z_gpu = pop.phenotypes().astype(np.float64)
        pop.close()
        cpu = {}
        for name, thr in (("all_cores", threads), ("single_core", 1)):
            orc = oracle.Oracle(T=w.T, fitness=fits[w.fitness], fit_param=w.fit_param, mu=w.mu, rho=w.rho,
                                bias=w.bias, p_neutral=w.p_neutral, q1=True, threads=thr, seed=7)
            orc.load_population(w.N, rows, pos, eff.reshape(-1))
            if name == "all_cores" and w.p_neutral < 1.0:
                err = np.abs(orc.phenotypes() - z_gpu)
                gpu["phenotype_error"] = {"max": float(err.max()), "mean": float(err.mean()),
                                          "max_abs_z": float(np.abs(z_gpu).max()),
                                          "note": "FP32-carried phenotypes after the whole run against the "
                                                  "FP64 sums of the same rows (the oracle's order)"}
            n = cpu_gens if thr > 1 else max(1, cpu_gens // 2)
            t0 = time.perf_counter()
            stages = {}
            for _ in range(n):
                orc.step_record(w.N)
                for k, v in orc.times().items():
                    stages[k] = stages.get(k, 0.0) + v
            dt = time.perf_counter() - t0
            orc.close()
            rate = 2.0 * w.N * n / dt
            cpu[name] = {"seq_gen_per_s": rate, "cores": thr, "generations": n, "s": dt, "stage_seconds": stages,
                         "derived_gbs": rate * 16.0 * info["W"] / 1e9}
        del rows
        out[key] = {"workload": w.name, "gpu": gpu, "cpu": cpu,
                    "cpu_sample": "oracle/clotho_oracle.cpp from the GPU run's final state (same rows, allele "
                                  "and effect tables), its own draws"}
    out["neutral_wf"]["note"] = "about 10 MB of rows: L2-resident, bound by launch and dependent latency, not HBM"
    return out


def single_core_rate(w, warmup=1, steps=2, N=None):
    """The reference's default thread count is the master thread alone (T=0,
    thread_count_parameter.hpp:22): the oracle on one core over a bounded sample
    of the workload (N=CPU_SAMPLE_N individuals, the same allele load and row
    width; the per-row cost does not depend on N)."""
    N = N or CPU_SAMPLE_N
    v, dt, info, _ = run_cpu_oracle(w, N, steps, warmup, 1)
    return {"value": v, "unit": UNIT, "cores": 1, "kind": "port", "derived_gbs": v * 16.0 * info["B"] / 1e9,
            "sample": (f"oracle/clotho_oracle.cpp on 1 thread (the reference's default T=0), N={N} "
                       f"individuals, same allele load (A={info['A']}, W={info['B']} words/row), {steps} "
                       f"generations after {warmup} warm-up, {dt:.1f} s")}


def reference_arm(args, rank):
    """The reference's CPU path (its restatement, oracle/clotho_oracle.cpp: the reference itself needs Boost,
    absent here) on this arm's own configuration: N=1e6 individuals with the same pre-seeded allele load,
    every host thread, K generations after W warm-up; beside it the single-core rate."""
    from clotho_gb300.workloads import LARGE_N
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    w = LARGE_N
    N = REF_N or getattr(args, "n", None) or w.N
    t_setup = time.perf_counter()
    v, dt, info, stages = run_cpu_oracle(w, N, args.steps, args.warmup, threads)
    t_setup = time.perf_counter() - t_setup - dt
    sample = (f"CPU restatement of the reference path (oracle/clotho_oracle.cpp) on {threads} host threads, the "
              f"full workload: N={N} individuals ({2 * N} rows), pre-seeded allele load (A={info['A']}, "
              f"W={info['B']} words/row), {args.steps} generations after {args.warmup} warm-up")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": {"workload": w.name, "N": N, "T": w.T, "A": info["A"], "W_live": info["B"], "rho": w.rho,
                       "mu": w.mu, "fitness": w.fitness, "threads": threads, "same_config": N == w.N},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                             "stage_seconds": stages, "setup_seconds": t_setup,
                             "derived_gbs": v * 16.0 * info["B"] / 1e9},
            "single_core": single_core_rate(w, N=min(CPU_SAMPLE_N, N)),
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def phase_breakdown(pop, N, warmup, steps):
    """Where the fused generation kernel spends its time: the profiling build
    clocks each row's phases (SM cycles summed over warps) over `steps`
    generations after `warmup` plain ones.  Shares are of the warps' resident
    cycles; the clock reads and their registers slow that build by a few percent."""
    for _ in range(warmup):
        pop.simulate_philox(N)
    pop.sync()
    pop.profile(True, phases=True)
    for _ in range(steps):
        pop.simulate_philox(N)
    pop.sync()
    ph = pop.phase_clocks()
    ms, launches, rows, _ = pop.kernel_time()
    pop.profile(False)
    warp = max(ph["warp_cycles"], 1)
    nc, nx = max(ph["copy_rows"], 1), max(ph["xo_rows"], 1)
    per_row = {
        "copy": {k: ph["copy_" + k] / nc for k in ("setup", "body", "phenotype")},
        "crossover": {k: ph["xo_" + k] / nx for k in ("setup", "mask", "body", "gather", "phenotype")},
    }
    share = {
        "copy_rows": (ph["copy_setup"] + ph["copy_body"] + ph["copy_phenotype"]) / warp,
        "xo_setup": ph["xo_setup"] / warp,
        "xo_mask": ph["xo_mask"] / warp,
        "xo_stream": (ph["xo_body"] - ph["xo_gather"]) / warp,
        "xo_gather": ph["xo_gather"] / warp,
        "xo_phenotype": ph["xo_phenotype"] / warp,
        "long_rows": ph["long_cycles"] / warp,
    }
    share["outside_rows"] = 1.0 - sum(share.values())
    return {"phase_clocks": True, "N": N, "generations": steps, "rows": {"copy": ph["copy_rows"],
            "crossover": ph["xo_rows"], "long": ph["long_rows"], "profiled": rows},
            "kernel_ms_per_gen": ms / max(launches, 1), "warps": ph["warps"],
            "cycles_per_row": per_row, "share_of_warp_cycles": {k: round(v, 4) for k, v in share.items()},
            "raw": ph}


def batch_kernels(cg, warmup, steps):
    """The batched measurement's 256 populations (the same job list and tuned-size items), stepped eagerly
    one generation at a time, for launch lists of a batched step."""
    from clotho_gb300 import serving
    jobs = serving.synthetic_jobs(256, rate=1e9, seed=11, N_range=(1_000, 200_000), G_range=(100, 100))
    b = cg.Batch([j.desc() for j in jobs])
    b.init()
    b.set_tuning(rows_per_item=1024)
    for _ in range(warmup + steps):
        b.step()
    b.sync()
    errs = sum(b.info(i)["device_error"] != 0 for i in range(len(jobs)))
    return {"batch_kernels": True, "populations": len(jobs), "generations": warmup + steps, "device_errors": errs,
            "max_row_words": max(b.info(i)["W"] for i in range(len(jobs)))}


def free_port() -> int:
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def relaunch_as_ranks(gpus: int) -> int:
    """`bench.py --gpus N` started without a launcher: start its N replica processes (one per GPU) on this
    node with the environment torchrun gives its ranks, and return the first nonzero exit status."""
    port = str(free_port())
    procs = []
    for r in range(gpus):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(gpus), LOCAL_WORLD_SIZE=str(gpus),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=port)
        procs.append(subprocess.Popen([sys.executable, os.path.abspath(__file__), *sys.argv[1:]], env=env))
    codes = [p.wait() for p in procs]
    return next((c for c in codes if c), 0)


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_as_ranks(args.gpus))
    rank, world, local = dist_env()
    if args.impl == "reference":
        reference_arm(args, rank)
        return
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = Dist(world)

    import numpy as np
    import clotho_gb300 as cg
    from clotho_gb300.workloads import LARGE_N, seeded_start

    if args.batch_kernels:
        print(json.dumps(batch_kernels(cg, args.warmup, args.steps)))
        return
    if args.c4_waves:
        print(json.dumps(c4_waves()))
        return
    if args.qtl_kernel:
        from clotho_gb300.workloads import QTL_SELECTION as q
        pop = cg.Population(q.N, q.max_alleles, q.T, fitness=q.fitness, fit_param=q.fit_param, mu=q.mu, rho=q.rho,
                            bias=q.bias, p_neutral=q.p_neutral, seed=20261203, max_fixed=1 << 20)
        pop.init(q.N)
        for _ in range(args.qtl_kernel + args.warmup + args.steps):
            pop.simulate_philox(q.N)
        pop.sync()
        pop.check()
        print(json.dumps({"qtl_kernel": True, "info": pop.info()}))
        return
    if args.configs_only:
        print(json.dumps({"configs": stated_configs(cg, os.cpu_count() or 1)}))
        return
    if args.batched_only:
        batched, serve = batched_and_serving()
        print(json.dumps({"batched": batched, "serving": serve}))
        return

    w = LARGE_N
    N = args.n or w.N
    pop = make_population(cg, w, N)
    pos, eff, thr = seeded_start(w, N=N)
    pop.seed_population(N, pos, eff, thr, 99)

    if args.phase_clocks:
        print(json.dumps(phase_breakdown(pop, N, args.warmup, args.steps)))
        return

    if args.kernel_only:
        for _ in range(args.warmup + args.steps):
            pop.simulate_philox(N)
        pop.sync()
        pop.check()
        print(json.dumps({"kernel_only": True, "N": N, "info": pop.info()}))
        return

    for _ in range(args.warmup):
        pop.simulate_philox(N)
    pop.sync()
    pop.check()

    # ---- timed region: K device-resident generations (graph replay)
    clocks = ClockSampler(0 if world == 1 else local)
    clocks.start()
    dist.barrier()
    pop.sync()
    l0 = pop.launches
    pop.timer_begin()
    pop.run_philox(N, args.steps)
    ms = pop.timer_end()
    pop.sync()
    dist.barrier()
    launches = pop.launches - l0
    ms = dist.max(ms)
    clk = clocks.stop()
    info = pop.info()
    pop.check()
    value = 2.0 * N * args.steps * world / (ms / 1e3)

    # ---- dominant kernel: CUDA events around each fused generation launch
    pop.profile(True)
    for _ in range(args.profile_gens):
        pop.simulate_philox(N)
    kms, nl, rows_done, words_done = pop.kernel_time()
    pop.profile(False)
    avg_ms = kms / max(nl, 1)
    bytes_per_launch = 16.0 * words_done / max(nl, 1)       # 16 B per (row, live word)
    w_live = words_done / max(rows_done, 1)
    achieved = bytes_per_launch / (avg_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    traffic = ncu_traffic()
    # DRAM bytes per (row, live word) from one ncu capture of this kernel on a smaller
    # population of the same workload (profiles/), scaled to this launch's rows x words
    per_word = (traffic or {}).get("dram_bytes_per_row_word")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": per_word * words_done / max(nl, 1) if per_word else None,
                "peak_kind": f"of {peak_kind}", "kernel": "k_generation", "kernel_ms": avg_ms,
                "algorithmic_bytes_per_launch": bytes_per_launch, "W_live": w_live,
                "step_share": (avg_ms * args.steps) / ms if ms else None}

    # ---- end to end through the C-ABI tape call with host buffers
    e2e = None
    if not args.no_e2e:
        rng = np.random.default_rng(1)
        tapes, keep = [], []
        for _ in range(2):
            t = cg.neutral_tape(rng, N, w.mu, w.rho, w.bias, w.T, p_neutral=w.p_neutral)
            pt, ptr = pinned_tape(cg, t)
            tapes.append(pt)
            keep.append(ptr)
        h2d = tapes[0].nbytes + 8
        pop.simulate(tapes[0])
        pop.info()
        dist.barrier()
        pop.sync()
        # every step uploads its tape and reads back its status; the next step is issued before the
        # previous status is collected, so its tape upload overlaps the previous step's kernels
        t0 = time.perf_counter()
        pop.simulate(tapes[0])
        ticket = pop.info_request()
        for k in range(1, args.steps + 1):
            nxt = None
            if k < args.steps:
                pop.simulate(tapes[k % 2])
                nxt = pop.info_request()
            pop.info_wait(ticket)  # device->host read of step k-1's status (mean fitness)
            ticket = nxt
        dt = time.perf_counter() - t0
        dist.barrier()
        dt = dist.max(dt)
        pop.check()
        e2e = {"value": 2.0 * N * args.steps * world / dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": 80, "ms_per_step": 1e3 * dt / args.steps,
               "note": "tape call per generation (uniform-parent tape), wall clock around H2D + kernels + D2H; "
                       "each step's status read is collected after the next step is issued; the two tapes are "
                       "drawn on the host before the timed region and replayed, so host-side drawing of the "
                       "tape (the reference's serial RNG draws) is not in this number"}
        for ptr in keep:
            cg.capi.load().clotho_host_free(ptr)
        if rank == 0 and world == 1:
            e2e["drop_in_host_draws"] = drop_in_rate(N, w)

    # ---- CPU baseline (rank 0, N=1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, dt, oinfo, stages = run_cpu_oracle(w, CPU_LEG_N, 4, 1, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": (f"oracle/clotho_oracle.cpp on {threads} host threads, N={CPU_LEG_N} individuals, same "
                          f"allele load (A={oinfo['A']}, W={oinfo['B']}), 4 generations after 1 warm-up, "
                          f"{dt:.1f} s"),
               "stage_seconds": stages, "single_core": single_core_rate(w),
               "derived_gbs": v * 16.0 * oinfo["B"] / 1e9,
               "derived_gbs_note": "seq-gen/s x 16 B x the row width: the GPU roofline's algorithmic basis"}

    batched = serve = None
    if rank == 0 and world == 1 and not args.no_batched:
        pop.close()
        batched, serve = batched_and_serving()

    configs = None
    if rank == 0 and world == 1 and not args.no_configs:
        pop.close()
        configs = stated_configs(cg, os.cpu_count() or 1)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "u64", "data": "synthetic",
                "config": {"workload": w.name, "N": N, "T": w.T, "A": info["A"], "W_live": info["W"],
                           "rho": w.rho, "mu": w.mu, "rng": "device Philox-4x32-10", "fitness": w.fitness,
                           "parallelism": "replicas" if world > 1 else "single",
                           "l2": "inputs larger than L2 (rows 16 GB per population)"},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
                "batched": batched, "serving": serve, "configs": configs}
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
