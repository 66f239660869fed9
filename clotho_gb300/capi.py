"""ctypes declarations of include/clotho_gpu.h.

Loading fails loudly when the library has not been built or does not export
the declared symbols; there is no CPU fallback anywhere in the package.
"""
from __future__ import annotations

import ctypes as C
import os

from . import builder as _build

vp = C.c_void_p
u32 = C.c_uint32
u64 = C.c_uint64
i32 = C.c_int32


class Tuning(C.Structure):
    _fields_ = [("rows_per_item", u32), ("narrow_build", u32), ("row_blocks_per_sm", u32)]


class Desc(C.Structure):
    _fields_ = [
        ("max_individuals", u32), ("max_alleles", u32), ("traits", u32), ("max_events", u32),
        ("max_mutations", u32), ("max_fixed", u32), ("fitness", i32), ("flags", u32),
        ("fit_param", C.c_double), ("mu", C.c_double), ("rho", C.c_double), ("bias", C.c_double),
        ("p_neutral", C.c_double), ("eff_mean", C.c_double), ("eff_sigma", C.c_double),
        ("seed", u64),
    ]


class GenTape(C.Structure):
    _fields_ = [
        ("N", u32), ("M", u32), ("pairs", vp), ("swap", vp), ("ev_off", vp), ("ev_pos", vp),
        ("mut_seq", vp), ("mut_pos", vp), ("mut_eff", vp),
    ]


class Info(C.Structure):
    _fields_ = [(n, u32) for n in (
        "generation", "N", "A", "W", "fixed_count", "lost_count", "free_count", "variable_count",
        "fixed_total", "last_M", "all_neutral", "device_error")] + [("mean_fitness", C.c_double)]


class Pairwise(C.Structure):
    _fields_ = [("count", C.c_uint64), ("total", C.c_uint64), ("min", u32), ("max", u32),
                ("mean", C.c_double), ("variance", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("segregating", u32), ("fixed_now", u32), ("mean_fitness", C.c_double),
                ("mean_phenotype", C.c_double * 4), ("heterozygosity", C.c_double)]


# name -> (restype, argtypes); every entry point declared in include/clotho_gpu.h
SIGNATURES = {
    "clotho_create": (C.c_int, [C.POINTER(Desc), C.POINTER(vp)]),
    "clotho_destroy": (C.c_int, [vp]),
    "clotho_last_error": (C.c_char_p, [vp]),
    "clotho_footprint": (C.c_size_t, [vp]),
    "clotho_footprint_for": (C.c_size_t, [C.POINTER(Desc)]),
    "clotho_sync": (C.c_int, [vp]),
    "clotho_init": (C.c_int, [vp, u32]),
    "clotho_seed_population": (C.c_int, [vp, u32, u32, vp, vp, vp, u64]),
    "clotho_load_population": (C.c_int, [vp, u32, u32, vp, vp, vp]),
    "clotho_generation_tape": (C.c_int, [vp, C.POINTER(GenTape)]),
    "clotho_generation_philox": (C.c_int, [vp, u32]),
    "clotho_run_philox": (C.c_int, [vp, u32, u32]),
    "clotho_begin_generation": (C.c_int, [vp, u32, u32]),
    "clotho_free_space": (C.c_int, [vp, vp]),
    "clotho_set_pairs": (C.c_int, [vp, vp]),
    "clotho_select": (C.c_int, [vp, vp]),
    "clotho_crossover": (C.c_int, [vp, vp, vp, vp]),
    "clotho_mutate": (C.c_int, [vp, vp, vp, vp]),
    "clotho_phenotype": (C.c_int, [vp]),
    "clotho_fitness": (C.c_int, [vp]),
    "clotho_end_generation": (C.c_int, [vp]),
    "clotho_get_info": (C.c_int, [vp, C.POINTER(Info)]),
    "clotho_info_request": (C.c_int, [vp, C.POINTER(u32)]),
    "clotho_info_wait": (C.c_int, [vp, u32, C.POINTER(Info)]),
    "clotho_get_rows": (C.c_int, [vp, vp, C.c_size_t]),
    "clotho_get_alleles": (C.c_int, [vp, vp, vp, vp]),
    "clotho_get_fixed": (C.c_int, [vp, vp, vp, vp]),
    "clotho_get_free": (C.c_int, [vp, vp]),
    "clotho_get_genome_traits": (C.c_int, [vp, vp]),
    "clotho_get_phenotypes": (C.c_int, [vp, vp]),
    "clotho_get_fitness": (C.c_int, [vp, vp]),
    "clotho_get_pairs": (C.c_int, [vp, vp]),
    "clotho_stats_compute": (C.c_int, [vp, C.POINTER(Stats), vp, u32]),
    "clotho_margins": (C.c_int, [vp, vp, vp]),
    "clotho_set_stream": (C.c_int, [vp, vp]),
    "clotho_run_philox_schedule": (C.c_int, [vp, vp, u32]),
    "clotho_pairwise_difference": (C.c_int, [vp, vp, u32, vp, C.POINTER(Pairwise)]),
    "clotho_pop_pairwise_difference": (C.c_int, [vp, u32, vp, u32, vp, C.POINTER(Pairwise)]),
    "clotho_pop_margins": (C.c_int, [vp, u32, vp, vp]),
    "clotho_snapshot_size": (C.c_size_t, [vp]),
    "clotho_snapshot": (C.c_int, [vp, vp, C.c_size_t]),
    "clotho_restore": (C.c_int, [vp, vp, C.c_size_t]),
    "clotho_profile": (C.c_int, [vp, C.c_int]),
    "clotho_phase_clocks": (C.c_int, [vp, C.POINTER(C.c_uint64), C.c_uint32]),
    "clotho_kernel_time": (C.c_int, [vp, C.POINTER(C.c_double), C.POINTER(u32), C.POINTER(u64), C.POINTER(u64)]),
    "clotho_timer_begin": (C.c_int, [vp]),
    "clotho_timer_end": (C.c_int, [vp, C.POINTER(C.c_double)]),
    "clotho_launch_count": (u64, [vp]),
    "clotho_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(vp)]),
    "clotho_batch_create": (C.c_int, [vp, u32, C.POINTER(vp)]),
    "clotho_pop_count": (u32, [vp]),
    "clotho_pop_add": (C.c_int, [vp, C.POINTER(Desc), C.POINTER(u32)]),
    "clotho_pop_remove": (C.c_int, [vp, u32]),
    "clotho_pop_init": (C.c_int, [vp, u32, u32]),
    "clotho_pop_info": (C.c_int, [vp, u32, C.POINTER(Info)]),
    "clotho_pop_info_request": (C.c_int, [vp, u32, C.POINTER(u32)]),
    "clotho_pop_rows": (C.c_int, [vp, u32, vp, C.c_size_t]),
    "clotho_pop_stats": (C.c_int, [vp, u32, C.POINTER(Stats), vp, u32]),
    "clotho_batch_generation_philox": (C.c_int, [vp, vp]),
    "clotho_batch_run_philox": (C.c_int, [vp, vp, u32]),
    "clotho_set_rows_per_item": (C.c_int, [vp, u32]),
    "clotho_set_copy_wait_limit": (C.c_int, [vp, u32]),
    "clotho_set_tuning": (C.c_int, [vp, vp]),
    "clotho_pop_count_columns": (C.c_int, [vp, u32, C.c_int]),
    "clotho_get_tuning": (C.c_int, [vp, vp]),
    "clotho_mem_info": (C.c_int, [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "clotho_free_space_noalloc": (C.c_int, [vp, u32, u32, u32, vp, vp, vp]),
    "clotho_host_free": (C.c_int, [vp]),
}

_lib = None


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load libclotho_gpu.so; raises if it is missing or incomplete."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: run clotho_gb300.build.build()")
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)  # AttributeError if a declared symbol is not exported
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
