"""The numpy restatement of the device's draw rules (oracle/device_draws.py), on the CPU.

Philox-4x32-10 is pinned to the known-answer vectors published with the
Random123 library (counter, key) -> output; the prefix-sum restatement is
checked against exact sums; the samplers against their laws.  The GPU tests
(tests/test_gpu_device_draws.py) then hold the device to this restatement.
"""
import math

import numpy as np

from oracle import device_draws as dd


def test_philox_known_answer_vectors():
    cases = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in cases:
        got = dd.philox4x32(*[np.uint64(c) for c in ctr], key[0] | (key[1] << 32))
        assert tuple(int(x) for x in got) == want


def test_philox_vectorised_equals_scalar():
    k = np.arange(1000, dtype=np.uint64)
    vec = dd.philox4x32(k, 3, 17, dd.STREAM_SELECT, 0x123456789)
    for i in (0, 1, 500, 999):
        one = dd.philox4x32(np.uint64(i), 3, 17, dd.STREAM_SELECT, 0x123456789)
        assert all(int(v[i]) == int(o) for v, o in zip(vec, one))


def test_uniforms_are_53_bit_and_in_range():
    u = dd.u01(np.array([0, 0xFFFFFFFF, 0x80000000], np.uint64), np.array([0, 0xFFFFFFFF, 0], np.uint64))
    assert u[0] == 0.0 and u[1] == 1.0 - 2.0 ** -53 and u[2] == 0.5


def test_prefix_sum_restatement():
    rng = np.random.default_rng(3)
    for N in (1, 31, 4096, 4097, 10_000, 70_001):
        fit = rng.random(N) * 1e-3 + rng.integers(0, 2, N)
        cdf, total, same = dd.fitness_prefix(fit)
        ref = np.cumsum(fit, dtype=np.float64)
        # a different association order: equal up to a few ulps of the running sum
        assert np.all(np.abs(cdf - ref) <= 64 * np.finfo(np.float64).eps * ref[-1])
        assert abs(total - math.fsum(fit)) <= 64 * np.finfo(np.float64).eps * total
        assert np.all(np.diff(cdf) >= 0.0) and same == (N == 1)
    # integers sum exactly in any order
    fit = rng.integers(0, 5, 12_345).astype(np.float64)
    cdf, total, _ = dd.fitness_prefix(fit)
    assert np.array_equal(cdf, np.cumsum(fit)) and total == fit.sum()


def test_selection_restatement_follows_fitness():
    rng = np.random.default_rng(5)
    fit = rng.random(2000) ** 4
    ids, uniform, _, _ = dd.select_parents(fit, 50_000, 9, 77)
    assert not uniform and ids.size == 100_000 and ids.max() < 2000
    counts = np.bincount(ids, minlength=2000)
    exp = 100_000 * fit / fit.sum()
    top = np.argsort(exp)[-200:]
    assert abs(counts[top].sum() - exp[top].sum()) < 5 * math.sqrt(exp[top].sum())
    ids, uniform, _, _ = dd.select_parents(np.full(300, 0.25), 10_000, 9, 77)
    assert uniform and abs(np.bincount(ids, minlength=300).std() - math.sqrt(20_000 / 300)) < 3


def test_poisson_and_gamete_draws():
    u = np.random.default_rng(1).random(200_000)
    for lam in (0.01, 1.0, 5.0):
        k = dd.poisson_inv(u, lam, math.exp(-lam))
        assert abs(k.mean() - lam) < 5 * math.sqrt(lam / u.size) + 1e-4
        assert abs(k.var() - lam) < 0.05 * lam + 1e-3
    E, swap, off, pos = dd.gamete_draws(4000, 2, 11, 5.0, 0.3, True, math.exp(-5.0))
    assert E[1::2].sum() == 0 and off[-1] == E.sum() == pos.size
    assert abs(swap.mean() - 0.3) < 0.05 and pos.min() >= 0.0 and pos.max() < 1.0
    seq, mp = dd.mutation_draws(4000, 2, 11, 0.1, math.exp(-0.1))
    assert np.all(np.diff(seq.astype(np.int64)) >= 0) and abs(seq.size - 400) < 80 and mp.size == seq.size
    e = dd.mutation_effects(20_000, 2, 2, 11, 0.25, 0.0, 1.0)
    assert abs((e == 0).mean() - 0.25) < 0.02
    nz = e[e != 0]
    assert abs(nz.mean()) < 0.03 and abs(nz.std() - 1.0) < 0.03
