"""clotho_gb300 -- GB300-native (sm_103a) engine for the per-generation hot
path of putnampp/clotho.

The compute lives in libclotho_gpu.so (C-ABI, include/clotho_gpu.h).  This
module is the Python mirror of the reference's engine and stage policies
(examples/QTLSim/engine_batched_task.hpp:70-373) over that ABI; the C++
mirror is clotho_gb300/cpp/clotho_policies.hpp.  There is no CPU fallback:
every call goes to the CUDA library and raises on any error.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .tape import GenTape, neutral_tape, load_tapes, save_tapes  # noqa: F401

__all__ = ["Population", "GenTape", "neutral_tape", "ClothoError", "FITNESS", "build"]

# fitness_toolkit registry keys (src/clotho/fitness/fitness_toolkit.cpp:50-78)
FITNESS = {"constant": 0, "gaussian": 1, "quadratic": 2, "gaussian_vs": 3}
FLAG_Q1 = 1

DEVICE_ERRORS = {1: "allele capacity exceeded", 2: "fixed table capacity exceeded",
                 4: "more than 128 device-drawn events in a gamete", 8: "tape parent index out of range",
                 16: "tape mutation row out of range", 32: "mutation capacity exceeded",
                 64: "all fitness values zero", 128: "a parent strand copy outlived the wait limit",
                 256: "a parent strand copy never landed (rows left unfinished)"}


class ClothoError(RuntimeError):
    pass


def build(force: bool = False) -> str:
    from . import builder
    return builder.build(force=force)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None and a.size else None


class Population:
    """One resident population on the GPU: the Engine<...,batched_task> state
    (two population_space_row bitsets, AlleleSpace, trait_space_vector, free
    space, fixed tables, phenotypes and fitness)."""

    def __init__(self, max_individuals: int, max_alleles: int, traits: int = 1, *, max_events: int | None = None,
                 max_mutations: int | None = None, max_fixed: int | None = None, fitness: str = "constant",
                 fit_param: float = 1.0, mu: float = 1e-4, rho: float = 1e-4, bias: float = 0.5,
                 p_neutral: float = 0.5, eff_mean: float = 0.0, eff_sigma: float = 1.0, seed: int = 1,
                 q1: bool = True):
        self.L = capi.load()
        S = 2 * max_individuals
        if max_events is None:
            max_events = int(S * rho + 10 * np.sqrt(S * rho + 1) + 64)
        if max_mutations is None:
            max_mutations = int(S * mu + 10 * np.sqrt(S * mu + 1) + 64)
        if max_fixed is None:
            max_fixed = max(1024, max_alleles)
        self.T = int(traits)
        self.desc = capi.Desc(max_individuals, max_alleles, traits, max_events, max_mutations, max_fixed,
                              FITNESS[fitness], FLAG_Q1 if q1 else 0, fit_param, mu, rho, bias, p_neutral,
                              eff_mean, eff_sigma, seed)
        h = C.c_void_p()
        rc = self.L.clotho_create(C.byref(self.desc), C.byref(h))
        if rc != 0:
            raise ClothoError(f"clotho_create failed ({rc})")
        self.h = h

    # ---- lifetime
    def close(self):
        if getattr(self, "h", None):
            self.L.clotho_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc: int, what: str):
        if rc != 0:
            msg = self.L.clotho_last_error(self.h)
            raise ClothoError(f"{what}: rc={rc}: {msg.decode() if msg else ''}")

    @property
    def footprint(self) -> int:
        return int(self.L.clotho_footprint(self.h))

    def sync(self):
        self._ck(self.L.clotho_sync(self.h), "sync")

    def set_stream(self, stream=None):
        """Run on the caller's CUDA stream (an integer handle, e.g.
        torch.cuda.Stream().cuda_stream); None returns to the context's own."""
        self._ck(self.L.clotho_set_stream(self.h, C.c_void_p(int(stream)) if stream else None), "set_stream")

    # ---- set-up
    def init(self, N0: int):
        self._ck(self.L.clotho_init(self.h, N0), "init")

    def seed_population(self, N: int, pos, eff, thr, seed: int):
        pos = np.ascontiguousarray(pos, np.float64)
        eff = np.ascontiguousarray(eff, np.float32)
        thr = np.ascontiguousarray(thr, np.uint32)
        self._ck(self.L.clotho_seed_population(self.h, N, len(pos), _ptr(pos), _ptr(eff), _ptr(thr), seed),
                 "seed_population")

    def load_population(self, N: int, rows, pos, eff):
        """Explicit start from rows in the reference layout (2N x ceil(A/512)*8 words)."""
        rows = np.ascontiguousarray(rows, np.uint64)
        pos = np.ascontiguousarray(pos, np.float64)
        eff = np.ascontiguousarray(eff, np.float32)
        self._ck(self.L.clotho_load_population(self.h, N, len(pos), _ptr(rows), _ptr(pos), _ptr(eff)),
                 "load_population")

    # ---- fused generation (Engine::simulate)
    def simulate(self, tape):
        t = tape if isinstance(tape, GenTape) else GenTape(tape.N, tape.M, tape.pairs, tape.swap, tape.ev_off,
                                                            tape.ev_pos, tape.mut_seq, tape.mut_pos, tape.mut_eff)
        t = t.contiguous()
        s = capi.GenTape(t.N, t.M, _ptr(t.pairs), _ptr(t.swap), _ptr(t.ev_off), _ptr(t.ev_pos), _ptr(t.mut_seq),
                         _ptr(t.mut_pos), _ptr(t.mut_eff))
        self._keep = t  # arrays must outlive the copy (the call waits for it anyway)
        self._ck(self.L.clotho_generation_tape(self.h, C.byref(s)), "generation_tape")

    def simulate_philox(self, N: int):
        self._ck(self.L.clotho_generation_philox(self.h, N), "generation_philox")

    def run_philox(self, N: int, G: int):
        self._ck(self.L.clotho_run_philox(self.h, N, G), "run_philox")

    def run_philox_schedule(self, sizes):
        """Device-drawn generations with N = sizes[g] offspring individuals in
        generation g (population growth), replayed from one CUDA graph."""
        n = np.ascontiguousarray(sizes, np.uint32)
        if n.size:
            self._ck(self.L.clotho_run_philox_schedule(self.h, _ptr(n), n.size), "run_philox_schedule")

    def run_growth(self, growth, G: int):
        """G generations whose sizes follow a growth model (clotho_gb300.growth)."""
        from . import growth as gr
        i = self.info()
        sizes = gr.schedule(growth, i["N"], i["generation"], G)
        self.run_philox_schedule(sizes)
        return sizes

    # ---- staged policies
    def begin_generation(self, N: int, M: int):
        self._ck(self.L.clotho_begin_generation(self.h, N, M), "begin_generation")

    def free_space(self):
        c = np.zeros(3, np.uint32)
        self._ck(self.L.clotho_free_space(self.h, _ptr(c)), "free_space")
        return int(c[0]), int(c[1]), int(c[2])

    def set_pairs(self, pairs):
        pairs = np.ascontiguousarray(pairs, np.uint32)
        self._ck(self.L.clotho_set_pairs(self.h, _ptr(pairs)), "set_pairs")

    def select(self, N: int):
        out = np.zeros(2 * N, np.uint32)
        self._ck(self.L.clotho_select(self.h, _ptr(out)), "select")
        return out

    def crossover(self, swap, ev_off, ev_pos):
        swap = np.ascontiguousarray(swap, np.uint8)
        ev_off = np.ascontiguousarray(ev_off, np.uint32)
        ev_pos = np.ascontiguousarray(ev_pos, np.float64)
        self._ck(self.L.clotho_crossover(self.h, _ptr(swap), _ptr(ev_off), _ptr(ev_pos)), "crossover")

    def mutate(self, mut_seq, mut_pos, mut_eff):
        mut_seq = np.ascontiguousarray(mut_seq, np.uint32)
        mut_pos = np.ascontiguousarray(mut_pos, np.float64)
        mut_eff = np.ascontiguousarray(mut_eff, np.float32)
        self._ck(self.L.clotho_mutate(self.h, _ptr(mut_seq), _ptr(mut_pos), _ptr(mut_eff)), "mutate")

    def phenotype(self):
        self._ck(self.L.clotho_phenotype(self.h), "phenotype")

    def evaluate_fitness(self):
        self._ck(self.L.clotho_fitness(self.h), "fitness")

    def end_generation(self):
        self._ck(self.L.clotho_end_generation(self.h), "end_generation")

    def simulate_staged(self, tape):
        """Engine::simulate driven stage by stage through the policy entry points."""
        t = tape
        self.begin_generation(t.N, t.M)
        self.free_space()
        self.set_pairs(t.pairs)
        self.crossover(t.swap, t.ev_off, t.ev_pos)
        self.mutate(t.mut_seq, t.mut_pos, t.mut_eff)
        self.phenotype()
        self.evaluate_fitness()
        self.end_generation()

    # ---- read-back
    def info(self) -> dict:
        i = capi.Info()
        self._ck(self.L.clotho_get_info(self.h, C.byref(i)), "get_info")
        return {n: getattr(i, n) for n, _ in capi.Info._fields_}

    def info_request(self) -> int:
        """Ticket for the status as of the work issued so far (returns at once)."""
        t = C.c_uint32()
        self._ck(self.L.clotho_info_request(self.h, C.byref(t)), "info_request")
        return t.value

    def info_wait(self, ticket: int) -> dict:
        """The status copied by info_request(ticket), once its copy has landed."""
        i = capi.Info()
        self._ck(self.L.clotho_info_wait(self.h, ticket, C.byref(i)), "info_wait")
        return {n: getattr(i, n) for n, _ in capi.Info._fields_}

    def set_tuning(self, rows_per_item: int = 0, narrow_build: int = 1, row_blocks_per_sm: int = 0):
        """Launch shapes (clotho_gb300.autotune); no result depends on them."""
        t = capi.Tuning(rows_per_item, narrow_build, row_blocks_per_sm)
        self._ck(self.L.clotho_set_tuning(self.h, C.byref(t)), "set_tuning")

    def count_columns(self, enable: bool = True):
        """Count every allele slot's carriers inside each later fused generation step, so stats() reads the
        counts instead of making a pass over the rows."""
        self._ck(self.L.clotho_pop_count_columns(self.h, 0, 1 if enable else 0), "count_columns")

    def set_copy_wait_limit(self, rounds: int):
        """try_wait rounds a copy row's bulk copy may take before the STALL flag is raised (0: default)."""
        self._ck(self.L.clotho_set_copy_wait_limit(self.h, rounds), "set_copy_wait_limit")

    def check(self):
        err = self.info()["device_error"]
        if err:
            raise ClothoError("device error: " + ", ".join(m for b, m in DEVICE_ERRORS.items() if err & b))

    def rows(self) -> np.ndarray:
        i = self.info()
        out = np.zeros((2 * i["N"], i["W"]), np.uint64)
        self._ck(self.L.clotho_get_rows(self.h, _ptr(out), out.size), "get_rows")
        return out

    def alleles(self):
        A = self.info()["A"]
        pos = np.zeros(A, np.float64)
        age = np.zeros(A, np.uint32)
        eff = np.zeros(A * self.T, np.float32)
        self._ck(self.L.clotho_get_alleles(self.h, _ptr(pos), _ptr(age), _ptr(eff)), "get_alleles")
        return pos, age, eff.reshape(A, self.T)

    def fixed(self):
        F = self.info()["fixed_total"]
        pos = np.zeros(F, np.float64)
        age = np.zeros(F, np.uint32)
        eff = np.zeros(F * self.T, np.float32)
        self._ck(self.L.clotho_get_fixed(self.h, _ptr(pos), _ptr(age), _ptr(eff)), "get_fixed")
        return pos, age, eff.reshape(F, self.T)

    def free_list(self) -> np.ndarray:
        n = self.info()["free_count"]
        out = np.zeros(n, np.uint32)
        self._ck(self.L.clotho_get_free(self.h, _ptr(out)), "get_free")
        return out

    def genome_traits(self) -> np.ndarray:
        S = 2 * self.info()["N"]
        out = np.zeros(S * self.T, np.float64)
        self._ck(self.L.clotho_get_genome_traits(self.h, _ptr(out)), "get_genome_traits")
        return out.reshape(S, self.T)

    def phenotypes(self) -> np.ndarray:
        N = self.info()["N"]
        out = np.zeros(N * self.T, np.float64)
        self._ck(self.L.clotho_get_phenotypes(self.h, _ptr(out)), "get_phenotypes")
        return out.reshape(N, self.T)

    def fitness(self) -> np.ndarray:
        N = self.info()["N"]
        out = np.zeros(N, np.float64)
        self._ck(self.L.clotho_get_fitness(self.h, _ptr(out)), "get_fitness")
        return out

    def pairs(self) -> np.ndarray:
        """Parent individual of each of the last generation's 2N gametes (gametes 2k and 2k+1 make
        individual k), whichever call made that generation: a tape, device draws or the staged calls."""
        N = self.info()["N"]
        out = np.zeros(2 * N, np.uint32)
        self._ck(self.L.clotho_get_pairs(self.h, _ptr(out)), "get_pairs")
        return out

    def margins(self):
        """(col_counts[A], row_counts[2N]): sequences per allele slot, alleles per sequence."""
        i = self.info()
        col = np.zeros(max(1, i["A"]), np.uint32)
        row = np.zeros(max(1, 2 * i["N"]), np.uint32)
        self._ck(self.L.clotho_margins(self.h, _ptr(col), _ptr(row)), "margins")
        return col[: i["A"]], row[: 2 * i["N"]]

    def allele_frequency_log(self) -> dict:
        """The reference's `allele_frequency` log entry for the whole population."""
        from . import logs
        col, row = self.margins()
        return logs.allele_frequency(col, row, 2 * self.info()["N"])

    def pairwise_difference(self, sample=None, n: int | None = None, distances: bool = False) -> dict:
        """Pairwise differences over sampled rows (all pairs i < j): the
        reference's min / max / mean / median / variance plus count and total.
        sample: row indices (default rows 0..n-1, n default 2N).  The median
        needs the distances, so it is reported when distances=True."""
        if sample is not None:
            sample = np.ascontiguousarray(sample, np.uint32)
            n = sample.size
        elif n is None:
            n = 2 * self.info()["N"]
        pw = capi.Pairwise()
        d = np.zeros(max(1, n * (n - 1) // 2), np.uint32) if distances else None
        self._ck(self.L.clotho_pairwise_difference(self.h, _ptr(sample), n, _ptr(d) if distances else None,
                                                    C.byref(pw)), "pairwise_difference")
        out = {"min": pw.min, "max": pw.max, "mean": pw.mean, "variance": pw.variance, "count": pw.count,
               "total": pw.total}
        if distances:
            d = d[: n * (n - 1) // 2]
            out["median"] = float(np.median(d)) if d.size else 0.0
            out["distances"] = d
        return out

    def write_ms(self, fp, sample=None, seeds=(0, 0, 0)):
        """Write the sampled rows (default: all) in Hudson's ms format; returns the slots written."""
        from . import ms
        pos, _, _ = self.alleles()
        return ms.write_ms(fp, self.rows(), pos, sample=sample, seeds=seeds)

    # ---- checkpoint / resume (between generations)
    def snapshot(self) -> bytes:
        n = int(self.L.clotho_snapshot_size(self.h))
        if n == 0:
            msg = self.L.clotho_last_error(self.h)
            raise ClothoError("snapshot: " + (msg.decode() if msg else "no snapshot can be taken now"))
        buf = np.empty(n, np.uint8)
        self._ck(self.L.clotho_snapshot(self.h, _ptr(buf), n), "snapshot")
        return buf.tobytes()

    def restore(self, data: bytes):
        buf = np.frombuffer(data, np.uint8).copy()
        self._ck(self.L.clotho_restore(self.h, _ptr(buf), buf.size), "restore")

    def save(self, path: str):
        with open(path, "wb") as f:
            f.write(self.snapshot())

    def load(self, path: str):
        with open(path, "rb") as f:
            self.restore(f.read())

    def stats(self, sfs_len: int = 0):
        st = capi.Stats()
        sfs = np.zeros(sfs_len, np.uint32) if sfs_len else None
        self._ck(self.L.clotho_stats_compute(self.h, C.byref(st), _ptr(sfs), sfs_len), "stats")
        d = {"segregating": st.segregating, "fixed_now": st.fixed_now, "mean_fitness": st.mean_fitness,
             "mean_phenotype": list(st.mean_phenotype)[: self.T], "heterozygosity": st.heterozygosity}
        if sfs is not None:
            d["sfs"] = sfs
        return d

    # ---- timing
    def profile(self, enable: bool, phases: bool = False):
        """Kernel events and row counts; phases=True also runs the generation
        kernel's phase-clock build (slower) for phase_clocks()."""
        self._ck(self.L.clotho_profile(self.h, (2 if phases else 1) if enable else 0), "profile")

    def kernel_time(self):
        ms = C.c_double()
        n = C.c_uint32()
        r = C.c_uint64()
        w = C.c_uint64()
        self._ck(self.L.clotho_kernel_time(self.h, C.byref(ms), C.byref(n), C.byref(r), C.byref(w)), "kernel_time")
        return ms.value, n.value, r.value, w.value

    PHASES = ("copy_rows", "copy_setup", "copy_body", "copy_phenotype", "xo_rows", "xo_setup", "xo_mask",
              "xo_body", "xo_gather", "xo_phenotype", "long_rows", "long_cycles", "warp_cycles", "warps")

    def phase_clocks(self) -> dict:
        """Per-phase SM cycles of the fused generation kernel since profile(True, phases=True)
        (summed over warps; the profiling build clocks each suffix-table row)."""
        out = (C.c_uint64 * len(self.PHASES))()
        self._ck(self.L.clotho_phase_clocks(self.h, out, len(self.PHASES)), "phase_clocks")
        return dict(zip(self.PHASES, (int(x) for x in out)))

    def timer_begin(self):
        self._ck(self.L.clotho_timer_begin(self.h), "timer_begin")

    def timer_end(self) -> float:
        ms = C.c_double()
        self._ck(self.L.clotho_timer_end(self.h, C.byref(ms)), "timer_end")
        return ms.value

    @property
    def launches(self) -> int:
        return int(self.L.clotho_launch_count(self.h))


def make_desc(N: int, max_alleles: int, traits: int = 1, *, mu: float = 1e-4, rho: float = 1e-4, bias: float = 0.5,
              p_neutral: float = 0.5, eff_mean: float = 0.0, eff_sigma: float = 1.0, fitness: str = "constant",
              fit_param: float = 1.0, seed: int = 1, q1: bool = True, max_events: int | None = None,
              max_mutations: int | None = None, max_fixed: int | None = None) -> capi.Desc:
    S = 2 * N
    if max_events is None:
        max_events = int(S * rho + 10 * np.sqrt(S * rho + 1) + 64)
    if max_mutations is None:
        max_mutations = int(S * mu + 10 * np.sqrt(S * mu + 1) + 64)
    if max_fixed is None:
        max_fixed = max(1024, max_alleles)
    return capi.Desc(N, max_alleles, traits, max_events, max_mutations, max_fixed, FITNESS[fitness],
                     FLAG_Q1 if q1 else 0, fit_param, mu, rho, bias, p_neutral, eff_mean, eff_sigma, seed)


def footprint_of(desc: capi.Desc) -> int:
    """Device bytes a population with this descriptor holds (admission control)."""
    return int(capi.load().clotho_footprint_for(C.byref(desc)))


def device_memory() -> tuple[int, int]:
    f, t = C.c_size_t(), C.c_size_t()
    rc = capi.load().clotho_mem_info(C.byref(f), C.byref(t))
    if rc != 0:
        raise ClothoError("clotho_mem_info failed")
    return f.value, t.value


class Batch:
    """Many resident populations in one context: every generation is one
    launch per stage over all of them, replayable from one CUDA graph."""

    def __init__(self, descs=()):
        self.L = capi.load()
        self.descs = list(descs)
        arr = (capi.Desc * max(1, len(self.descs)))(*self.descs)
        h = C.c_void_p()
        rc = self.L.clotho_batch_create(arr if self.descs else None, len(self.descs), C.byref(h))
        if rc != 0:
            raise ClothoError(f"clotho_batch_create failed ({rc})")
        self.h = h
        self.N = [d.max_individuals for d in self.descs]

    def _ck(self, rc, what):
        if rc != 0:
            msg = self.L.clotho_last_error(self.h)
            raise ClothoError(f"{what}: rc={rc}: {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "h", None):
            self.L.clotho_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return int(self.L.clotho_pop_count(self.h))

    def add(self, desc: capi.Desc, N0: int | None = None) -> int:
        idx = C.c_uint32()
        self._ck(self.L.clotho_pop_add(self.h, C.byref(desc), C.byref(idx)), "pop_add")
        self.descs.append(desc)
        self.N.append(desc.max_individuals if N0 is None else N0)
        self._ck(self.L.clotho_pop_init(self.h, idx.value, self.N[-1]), "pop_init")
        return idx.value

    def remove(self, index: int):
        self._ck(self.L.clotho_pop_remove(self.h, index), "pop_remove")
        del self.descs[index]
        del self.N[index]

    def init(self):
        for i, n in enumerate(self.N):
            self._ck(self.L.clotho_pop_init(self.h, i, n), "pop_init")

    def step(self):
        if not self.N:
            return
        n = np.ascontiguousarray(self.N, np.uint32)
        self._ck(self.L.clotho_batch_generation_philox(self.h, _ptr(n)), "batch_generation_philox")

    def run(self, G: int):
        if not self.N or G <= 0:
            return
        n = np.ascontiguousarray(self.N, np.uint32)
        self._ck(self.L.clotho_batch_run_philox(self.h, _ptr(n), G), "batch_run_philox")

    def run_schedule(self, sizes):
        """sizes[g][i]: offspring individuals of population i in generation g."""
        n = np.ascontiguousarray(sizes, np.uint32)
        if n.size:
            assert n.ndim == 2 and n.shape[1] == len(self.N)
            self._ck(self.L.clotho_run_philox_schedule(self.h, _ptr(n), n.shape[0]), "run_philox_schedule")
            self.N = [int(x) for x in n[-1]]

    def set_rows_per_item(self, rows: int):
        self._ck(self.L.clotho_set_rows_per_item(self.h, rows), "set_rows_per_item")

    def set_tuning(self, rows_per_item: int = 0, narrow_build: int = 1, row_blocks_per_sm: int = 0):
        """Launch shapes (clotho_gb300.autotune); no result depends on them."""
        t = capi.Tuning(rows_per_item, narrow_build, row_blocks_per_sm)
        self._ck(self.L.clotho_set_tuning(self.h, C.byref(t)), "set_tuning")

    def count_columns(self, i: int, enable: bool = True):
        """Population i counts its allele slots' carriers inside each later step (stats() then reads them)."""
        self._ck(self.L.clotho_pop_count_columns(self.h, i, 1 if enable else 0), "pop_count_columns")

    def tuning(self) -> dict:
        t = capi.Tuning()
        self._ck(self.L.clotho_get_tuning(self.h, C.byref(t)), "get_tuning")
        return {n: getattr(t, n) for n, _ in capi.Tuning._fields_}

    def set_stream(self, stream=None):
        """Run on the caller's CUDA stream (integer handle); None returns to the context's own."""
        self._ck(self.L.clotho_set_stream(self.h, C.c_void_p(int(stream)) if stream else None), "set_stream")

    def sync(self):
        self._ck(self.L.clotho_sync(self.h), "sync")

    def info(self, i: int) -> dict:
        inf = capi.Info()
        self._ck(self.L.clotho_pop_info(self.h, i, C.byref(inf)), "pop_info")
        return {n: getattr(inf, n) for n, _ in capi.Info._fields_}

    def info_request(self, i: int) -> int:
        t = C.c_uint32()
        self._ck(self.L.clotho_pop_info_request(self.h, i, C.byref(t)), "pop_info_request")
        return t.value

    def info_wait(self, ticket: int) -> dict:
        inf = capi.Info()
        self._ck(self.L.clotho_info_wait(self.h, ticket, C.byref(inf)), "info_wait")
        return {n: getattr(inf, n) for n, _ in capi.Info._fields_}

    def rows(self, i: int) -> np.ndarray:
        inf = self.info(i)
        out = np.zeros((2 * inf["N"], inf["W"]), np.uint64)
        self._ck(self.L.clotho_pop_rows(self.h, i, _ptr(out), out.size), "pop_rows")
        return out

    def stats(self, i: int, sfs_len: int = 0) -> dict:
        st = capi.Stats()
        sfs = np.zeros(sfs_len, np.uint32) if sfs_len else None
        self._ck(self.L.clotho_pop_stats(self.h, i, C.byref(st), _ptr(sfs), sfs_len), "pop_stats")
        d = {"segregating": st.segregating, "fixed_now": st.fixed_now, "mean_fitness": st.mean_fitness,
             "heterozygosity": st.heterozygosity}
        if sfs is not None:
            d["sfs"] = sfs
        return d

    def margins(self, i: int):
        """(col_counts[A], row_counts[2N]) of population i."""
        inf = self.info(i)
        col = np.zeros(max(1, inf["A"]), np.uint32)
        row = np.zeros(max(1, 2 * inf["N"]), np.uint32)
        self._ck(self.L.clotho_pop_margins(self.h, i, _ptr(col), _ptr(row)), "pop_margins")
        return col[: inf["A"]], row[: 2 * inf["N"]]

    @property
    def footprint(self) -> int:
        return int(self.L.clotho_footprint(self.h))

    @property
    def launches(self) -> int:
        return int(self.L.clotho_launch_count(self.h))

    def timer_begin(self):
        self._ck(self.L.clotho_timer_begin(self.h), "timer_begin")

    def timer_end(self) -> float:
        ms = C.c_double()
        self._ck(self.L.clotho_timer_end(self.h, C.byref(ms)), "timer_end")
        return ms.value
