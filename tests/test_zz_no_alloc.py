"""clotho_free_space_noalloc: the free-space analysis for callers that cannot
call cudaMalloc (their device memory belongs to another allocator, or they
may not allocate after start-up).  It reads rows the caller owns, writes the
free list and counts the caller owns, and keeps its working state in a fixed
array inside the library.  Checked through the C-ABI against the existing
entry point (clotho_free_space through a context) on two calls in a row with
different data, so state left by the first call must not leak into the
second.  Free lists and counts are integers: the bar is equality.

This file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu


def _rows(rng, S, A, fixed, lost):
    W = ((A + 511) // 512) * 8
    bits = rng.random((S, A)) < 0.3
    bits[:, fixed] = True
    bits[:, lost] = False
    padded = np.zeros((S, W * 64), bool)
    padded[:, :A] = bits
    return np.packbits(padded, axis=1, bitorder="little").view(np.uint64).reshape(S, W).copy(), W


def _existing(rows, N, A):
    import clotho_gb300 as cg
    pop = cg.Population(N, A, 1, mu=0.0, rho=0.0, p_neutral=1.0, max_events=16, max_mutations=16,
                        max_fixed=A + 64)
    pop.load_population(N, rows, np.linspace(0, 0.999, A), np.zeros(A, np.float32))
    pop.begin_generation(N, 0)
    counts = pop.free_space()
    free = pop.free_list()
    pop.close()
    return counts, free


def test_noalloc_matches_existing_entry_point_twice():
    if not gpu_available():
        pytest.skip("no CUDA device")
    torch = pytest.importorskip("torch")
    from clotho_gb300 import capi
    L = capi.load()
    rng = np.random.default_rng(17)
    cases = [(300, 3000, [5, 700, 2999], [1, 2, 3, 64, 1000]),   # first call: wider rows
             (90, 1100, [0, 513], [7, 8, 1099])]                 # second call: fewer rows, narrower
    for N, A, fixed, lost in cases:
        S = 2 * N
        rows, W = _rows(rng, S, A, fixed, lost)
        (nfix, nlost, nfree), want = _existing(rows, N, A)
        d_rows = torch.from_numpy(rows.view(np.int64)).cuda()
        d_free = torch.full((W * 64,), -1, dtype=torch.int32, device="cuda")
        d_counts = torch.full((3,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = L.clotho_free_space_noalloc(C.c_void_p(d_rows.data_ptr()), S, W, A, C.c_void_p(d_free.data_ptr()),
                                         C.c_void_p(d_counts.data_ptr()), None)
        torch.cuda.synchronize()
        assert rc == 0
        counts = d_counts.cpu().numpy().astype(np.int64)
        assert list(counts) == [nfix, nlost, nfree]
        got = d_free.cpu().numpy()[:nfree].astype(np.uint32)
        assert np.array_equal(got, want)
        assert nfix >= len(fixed) and set(fixed) <= set(got[:nfix].tolist())


def test_noalloc_rejects_widths_beyond_its_array():
    if not gpu_available():
        pytest.skip("no CUDA device")
    from clotho_gb300 import capi
    L = capi.load()
    dummy = C.c_void_p(16)   # never dereferenced: the size check fails first
    rc = L.clotho_free_space_noalloc(dummy, 2, 20000, 2_000_000, dummy, dummy, None)
    assert rc == -3  # CLOTHO_E_CAPACITY


def test_noalloc_matches_the_oracle_including_an_empty_population():
    # the same analysis against the CPU restatement directly (oracle.free_space), on rows with fixed,
    # lost and padding columns, and on S = 0 rows, which the reference reads as every slot of every
    # word lost (no row seeds the AND/OR, so the tail padding step never runs)
    if not gpu_available():
        pytest.skip("no CUDA device")
    torch = pytest.importorskip("torch")
    import oracle
    from clotho_gb300 import capi
    L = capi.load()
    rng = np.random.default_rng(29)
    for S, A, fixed, lost in [(64, 700, [3, 699], [0, 640]), (0, 700, [], []), (0, 64, [], []),
                              (2, 513, [512], [1])]:
        rows, W = _rows(rng, max(S, 1), A, fixed, lost)
        rows = rows[:S]
        want, nfix, nlost = oracle.free_space(rows.reshape(S, W), A)
        d_rows = torch.from_numpy(np.ascontiguousarray(rows).view(np.int64).reshape(-1)).cuda() if S else None
        d_free = torch.full((W * 64,), -1, dtype=torch.int32, device="cuda")
        d_counts = torch.full((3,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = L.clotho_free_space_noalloc(C.c_void_p(d_rows.data_ptr()) if S else None, S, W, A,
                                         C.c_void_p(d_free.data_ptr()), C.c_void_p(d_counts.data_ptr()), None)
        torch.cuda.synchronize()
        assert rc == 0
        counts = d_counts.cpu().numpy().astype(np.int64)
        assert list(counts) == [nfix, nlost, nfix + nlost], (S, A)
        assert np.array_equal(d_free.cpu().numpy()[:nfix + nlost].astype(np.uint32), want), (S, A)
        if S == 0:
            assert nfix == 0 and nlost == W * 64
