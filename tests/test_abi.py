"""The C-ABI library loads and exports every entry point that include/*.h
declares (no compute call: this runs without a GPU)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(clotho_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from clotho_gb300 import builder
    path = builder.build()
    lib = ctypes.CDLL(path)
    headers = glob.glob(os.path.join(ROOT, "include", "*.h"))
    assert headers
    names = [n for h in headers for n in declared(h)]
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    from clotho_gb300 import capi
    names = declared(os.path.join(ROOT, "include", "clotho_gpu.h"))
    assert set(names) <= set(capi.SIGNATURES), set(names) - set(capi.SIGNATURES)


def test_library_is_sm103a_only():
    # the build targets sm_103a alone (no PTX for other architectures)
    from clotho_gb300 import builder
    assert builder.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_footprint_query_needs_no_gpu():
    from clotho_gb300 import capi
    L = capi.load()
    d = capi.Desc(1000, 4096, 2, 1000, 100, 100, 0, 1, 1.0, 0.01, 0.01, 0.5, 0.5, 0.0, 1.0, 1)
    b = L.clotho_footprint_for(ctypes.byref(d))
    # two populations of 2000 rows x 64 words dominate
    assert b >= 2 * 2000 * 64 * 8


def test_suffix_tables_by_capacity_and_crossover_rate():
    # a population gets a suffix table (and its crossover plans) up to 65,536 allele slots, and up to 524,288
    # slots when its rho is at most 1 (chunk masks); otherwise the interval classifier, without them.  The
    # table alone is (A/64 + 1) x W words, so the footprints of rho 1 and rho 3 differ by at least that much
    # above 65,536 slots, and not at all up to 65,536 or above 524,288
    from clotho_gb300 import capi
    L = capi.load()

    def fp(A, rho):
        d = capi.Desc(1000, A, 1, 4096, 4096, 4096, 0, 1, 1.0, 0.01, rho, 0.5, 0.5, 0.0, 1.0, 1)
        return L.clotho_footprint_for(ctypes.byref(d))

    for A in (4096, 65_536, 600_000):
        assert fp(A, 1.0) == fp(A, 3.0), A
    for A in (70_000, 200_000, 524_288):
        W = (A + 511) // 512 * 8
        W = (W + 63) // 64 * 64
        slots = W * 64
        assert fp(A, 1.0) - fp(A, 3.0) >= (slots // 64 + 1) * W * 8, A


def test_oracle_exports_its_header():
    import oracle
    lib = ctypes.CDLL(oracle.build())
    text = open(os.path.join(ROOT, "oracle", "clotho_oracle.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = sorted(set(re.findall(r"\b(orc_[a-z_0-9]+)\s*\(", text)))
    assert names and all(hasattr(lib, n) for n in names)


def test_calls_without_a_context_or_with_bad_arguments_return_a_status():
    # argument checks come before any CUDA call, so they answer on a machine without a GPU too
    from clotho_gb300 import capi
    L = capi.load()
    E_ARG, E_CAPACITY = -1, -3
    info = capi.Info()
    assert L.clotho_destroy(None) == E_ARG
    assert L.clotho_last_error(None) == b"null context"
    assert L.clotho_get_info(None, ctypes.byref(info)) == E_ARG
    assert L.clotho_init(None, 10) == E_ARG
    assert L.clotho_generation_philox(None, 10) == E_ARG
    assert L.clotho_sync(None) == E_ARG
    assert L.clotho_set_stream(None, None) == E_ARG
    assert L.clotho_pop_count(None) == 0 and L.clotho_launch_count(None) == 0
    assert L.clotho_snapshot_size(None) == 0
    assert L.clotho_footprint_for(None) == 0
    out = ctypes.c_void_p()
    assert L.clotho_create(None, ctypes.byref(out)) == E_ARG
    d = capi.Desc(100, 1024, 1, 100, 100, 100, 0, 1, 1.0, 0.01, 0.01, 0.5, 0.5, 0.0, 1.0, 1)
    assert L.clotho_create(ctypes.byref(d), None) == E_ARG
    assert L.clotho_batch_create(None, 3, ctypes.byref(out)) == E_ARG           # descriptors missing
    many = (capi.Desc * 257)(*([d] * 257))
    assert L.clotho_batch_create(many, 257, ctypes.byref(out)) == E_ARG         # more than 256 populations
    # the allocation-free entry point: output pointers checked, then the width limit (16,384 words)
    counts = (ctypes.c_uint32 * 3)()
    free_list = (ctypes.c_uint32 * 8)()
    assert L.clotho_free_space_noalloc(None, 0, 0, 64, None, counts, None) == E_ARG
    assert L.clotho_free_space_noalloc(None, 0, 0, 64 * 16_384 + 1, free_list, counts, None) == E_CAPACITY
    assert L.clotho_free_space_noalloc(None, 4, 16, 64, free_list, counts, None) == E_ARG  # rows missing


def test_create_without_a_device_fails_cleanly():
    # no GPU here: clotho_create reports a CUDA error and hands back no context
    from tests.conftest import gpu_available
    if gpu_available():
        pytest.skip("a CUDA device is present")
    from clotho_gb300 import capi
    L = capi.load()
    d = capi.Desc(100, 1024, 1, 100, 100, 100, 0, 1, 1.0, 0.01, 0.01, 0.5, 0.5, 0.0, 1.0, 1)
    out = ctypes.c_void_p(1234)
    assert L.clotho_create(ctypes.byref(d), ctypes.byref(out)) == -2            # CLOTHO_E_CUDA
    assert not out.value
