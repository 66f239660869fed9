"""ctypes access to the CPU oracle (oracle/clotho_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA engine and the CPU
baseline timed by bench.py.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU legs import this module.  The product path never does.

The oracle restates putnampp/clotho's QTLSimMT per-generation step
(examples/QTLSim/engine_batched_task.hpp:163-345); see clotho_oracle.cpp for
the per-function citations.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

FIT_CONSTANT, FIT_GAUSSIAN, FIT_QUADRATIC, FIT_GAUSSIAN_VS = 0, 1, 2, 3
FLAG_Q1 = 1


class OrcTape(C.Structure):
    _fields_ = [
        ("N", C.c_uint32), ("M", C.c_uint32),
        ("pairs", C.c_void_p), ("swap", C.c_void_p), ("ev_off", C.c_void_p),
        ("ev_pos", C.c_void_p), ("mut_seq", C.c_void_p), ("mut_pos", C.c_void_p),
        ("mut_eff", C.c_void_p),
    ]


class OrcParams(C.Structure):
    _fields_ = [
        ("T", C.c_uint32), ("fitness", C.c_int32), ("fit_param", C.c_double),
        ("mu", C.c_double), ("rho", C.c_double), ("bias", C.c_double),
        ("p_neutral", C.c_double), ("eff_mean", C.c_double), ("eff_sigma", C.c_double),
        ("flags", C.c_uint32), ("threads", C.c_uint32), ("seed", C.c_uint64),
    ]


class OrcInfo(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in (
        "generation", "N", "S", "A", "B", "fixed_count", "lost_count", "free_count",
        "variable_count", "fixed_total", "all_neutral", "last_M")]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, portable flags)."""
    if force or not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "clotho_oracle.cpp"))):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        vp = C.c_void_p
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(OrcParams)]
        L.orc_destroy.argtypes = [vp]
        L.orc_init.argtypes = [vp, C.c_uint32]
        L.orc_seed_population.argtypes = [vp, C.c_uint32, C.c_uint32, vp, vp, vp, C.c_uint64]
        L.orc_load_population.argtypes = [vp, C.c_uint32, C.c_uint32, vp, vp, vp]
        L.orc_step_tape.argtypes = [vp, C.POINTER(OrcTape)]
        L.orc_step_tape.restype = C.c_int
        L.orc_step_record.argtypes = [vp, C.c_uint32]
        L.orc_step_record.restype = C.c_int
        L.orc_last_tape.argtypes = [vp, C.POINTER(OrcTape), C.POINTER(C.c_uint32)]
        L.orc_get_info.argtypes = [vp, C.POINTER(OrcInfo)]
        for n in ("orc_get_rows", "orc_get_free", "orc_get_genome_traits",
                  "orc_get_phenotypes", "orc_get_fitness", "orc_get_times"):
            getattr(L, n).argtypes = [vp, vp]
        L.orc_get_alleles.argtypes = [vp, vp, vp, vp]
        L.orc_get_fixed.argtypes = [vp, vp, vp, vp]
        L.orc_bit_walk.argtypes = [C.c_uint64, vp]
        L.orc_bit_walk.restype = C.c_uint32
        L.orc_free_space.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, vp, vp]
        L.orc_block_crossover.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, vp, C.c_uint32, vp, C.c_uint32]
        L.orc_block_crossover.restype = C.c_uint64
        L.orc_genome_weights.argtypes = [vp, C.c_uint32, vp, C.c_uint32, vp]
        L.orc_seed_hash.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
        L.orc_seed_hash.restype = C.c_uint32
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None and a.size else None


class Tape:
    """One generation of the event tape as numpy arrays (draw order)."""

    def __init__(self, N, M, pairs, swap, ev_off, ev_pos, mut_seq, mut_pos, mut_eff):
        self.N, self.M = int(N), int(M)
        self.pairs = np.ascontiguousarray(pairs, dtype=np.uint32)
        self.swap = np.ascontiguousarray(swap, dtype=np.uint8)
        self.ev_off = np.ascontiguousarray(ev_off, dtype=np.uint32)
        self.ev_pos = np.ascontiguousarray(ev_pos, dtype=np.float64)
        self.mut_seq = np.ascontiguousarray(mut_seq, dtype=np.uint32)
        self.mut_pos = np.ascontiguousarray(mut_pos, dtype=np.float64)
        self.mut_eff = np.ascontiguousarray(mut_eff, dtype=np.float32)

    def as_struct(self) -> OrcTape:
        return OrcTape(self.N, self.M, _p(self.pairs), _p(self.swap), _p(self.ev_off), _p(self.ev_pos),
                       _p(self.mut_seq), _p(self.mut_pos), _p(self.mut_eff))


class Oracle:
    def __init__(self, T=1, fitness=FIT_CONSTANT, fit_param=1.0, mu=0.01, rho=0.01, bias=0.5,
                 p_neutral=0.5, eff_mean=0.0, eff_sigma=1.0, q1=True, threads=1, seed=1):
        self.L = lib()
        self.T = T
        self.params = OrcParams(T, fitness, fit_param, mu, rho, bias, p_neutral, eff_mean, eff_sigma,
                                FLAG_Q1 if q1 else 0, threads, seed)
        self.h = self.L.orc_create(C.byref(self.params))

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self, N0):
        self.L.orc_init(self.h, N0)

    def seed_population(self, N, pos, eff, thr, seed):
        pos = np.ascontiguousarray(pos, np.float64)
        eff = np.ascontiguousarray(eff, np.float32)
        thr = np.ascontiguousarray(thr, np.uint32)
        self.L.orc_seed_population(self.h, N, len(pos), _p(pos), _p(eff), _p(thr), seed)

    def load_population(self, N, rows, pos, eff):
        rows = np.ascontiguousarray(rows, np.uint64)
        pos = np.ascontiguousarray(pos, np.float64)
        eff = np.ascontiguousarray(eff, np.float32)
        self.L.orc_load_population(self.h, N, len(pos), _p(rows), _p(pos), _p(eff))

    def step_tape(self, tape: Tape):
        s = tape.as_struct()
        rc = self.L.orc_step_tape(self.h, C.byref(s))
        if rc != 0:
            raise RuntimeError(f"oracle step failed: {rc}")

    def step_record(self, N) -> Tape:
        rc = self.L.orc_step_record(self.h, N)
        if rc != 0:
            raise RuntimeError(f"oracle step failed: {rc}")
        return self.last_tape()

    def last_tape(self) -> Tape:
        t = OrcTape()
        ev = C.c_uint32()
        self.L.orc_last_tape(self.h, C.byref(t), C.byref(ev))
        N, M, T = t.N, t.M, self.T

        def arr(ptr, n, dt):
            if n == 0 or not ptr:
                return np.zeros(0, dt)
            buf = (C.c_char * (n * np.dtype(dt).itemsize)).from_address(ptr)
            return np.frombuffer(buf, dtype=dt).copy()

        return Tape(N, M, arr(t.pairs, 2 * N, np.uint32), arr(t.swap, 2 * N, np.uint8),
                    arr(t.ev_off, 2 * N + 1, np.uint32), arr(t.ev_pos, ev.value, np.float64),
                    arr(t.mut_seq, M, np.uint32), arr(t.mut_pos, M, np.float64),
                    arr(t.mut_eff, M * T, np.float32))

    def info(self) -> dict:
        i = OrcInfo()
        self.L.orc_get_info(self.h, C.byref(i))
        return {n: getattr(i, n) for n, _ in OrcInfo._fields_}

    def rows(self):
        i = self.info()
        out = np.zeros((i["S"], i["B"]), np.uint64)
        if out.size:
            self.L.orc_get_rows(self.h, _p(out))
        return out

    def alleles(self):
        A = self.info()["A"]
        pos = np.zeros(A, np.float64)
        age = np.zeros(A, np.uint32)
        eff = np.zeros(A * self.T, np.float64)
        self.L.orc_get_alleles(self.h, _p(pos), _p(age), _p(eff))
        return pos, age, eff.reshape(A, self.T)

    def fixed(self):
        F = self.info()["fixed_total"]
        pos = np.zeros(F, np.float64)
        age = np.zeros(F, np.uint32)
        eff = np.zeros(F * self.T, np.float64)
        self.L.orc_get_fixed(self.h, _p(pos), _p(age), _p(eff))
        return pos, age, eff.reshape(F, self.T)

    def free_list(self):
        n = self.info()["free_count"]
        out = np.zeros(n, np.uint32)
        self.L.orc_get_free(self.h, _p(out))
        return out

    def genome_traits(self):
        S = self.info()["S"]
        out = np.zeros(S * self.T, np.float64)
        self.L.orc_get_genome_traits(self.h, _p(out))
        return out.reshape(S, self.T)

    def phenotypes(self):
        N = self.info()["N"]
        out = np.zeros(N * self.T, np.float64)
        self.L.orc_get_phenotypes(self.h, _p(out))
        return out.reshape(N, self.T)

    def fitness(self):
        N = self.info()["N"]
        out = np.zeros(N, np.float64)
        self.L.orc_get_fitness(self.h, _p(out))
        return out

    def times(self):
        out = np.zeros(6, np.float64)
        self.L.orc_get_times(self.h, _p(out))
        return dict(zip(("fixed", "crossover", "mutate", "phenotypes", "fitness", "total"), out.tolist()))


def bit_walk(w: int):
    idx = np.zeros(64, np.uint32)
    n = lib().orc_bit_walk(C.c_uint64(w), _p(idx))
    return idx[:n].tolist()


def free_space(rows: np.ndarray, A: int, threads: int = 1):
    rows = np.ascontiguousarray(rows, np.uint64)
    S, B = rows.shape
    out = np.zeros(max(A, B * 64), np.uint32)
    counts = np.zeros(3, np.uint32)
    lib().orc_free_space(_p(rows), S, B, A, threads, _p(out), _p(counts))
    return out[: counts[2]], int(counts[0]), int(counts[1])


def block_crossover(top, bottom, offset, positions, events):
    positions = np.ascontiguousarray(positions, np.float64)
    events = np.ascontiguousarray(events, np.float64)
    return int(lib().orc_block_crossover(C.c_uint64(top), C.c_uint64(bottom), offset, _p(positions),
                                         len(positions), _p(events), len(events)))


def genome_weights(row, w, T):
    row = np.ascontiguousarray(row, np.uint64)
    w = np.ascontiguousarray(w, np.float64)
    out = np.zeros(T, np.float64)
    lib().orc_genome_weights(_p(row), len(row), _p(w), T, _p(out))
    return out


def seed_hash(seed, row, slot):
    return int(lib().orc_seed_hash(C.c_uint64(seed), row, slot))
