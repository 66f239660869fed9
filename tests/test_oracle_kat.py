"""Known-answer tests of the CPU oracle, restated from the reference's own unit
tests on the population_space_row layout (the tests target the older
genetic_space API; the fixtures and expected values are theirs).

  free space   unittest/data_spaces/free_space_test.cpp:30-66
  crossover    unittest/data_spaces/crossover_test.cpp:37-111
  phenotype    unittest/data_spaces/linear_phenotype_test.cpp:47-137
  mutation     unittest/data_spaces/mutation_test.cpp:42-75
  bit walker   unittest/utility/debruijn_bit_walker_test.cpp:24-106
  popcount     unittest/utility/popcount_test.cpp:21-41
"""
import numpy as np
import pytest

import oracle


def rows_with(S, A, bits):
    B = ((A + 511) // 512) * 8
    r = np.zeros((S, B), np.uint64)
    for s, a in bits:
        r[s, a // 64] |= np.uint64(1) << np.uint64(a % 64)
    return r


def bit(rows, s, a):
    return bool((int(rows[s, a // 64]) >> (a % 64)) & 1)


# ---- free_space_test.cpp:30-66: 200 alleles x 22 genomes; allele 101 set in
# every genome, allele 33 set in genome 2  ->  fixed 1, lost 198, free 199.
def test_free_space_fixture():
    S, A = 22, 200
    rows = rows_with(S, A, [(i, 101) for i in range(S)] + [(2, 33)])
    free, nfix, nlost = oracle.free_space(rows, A)
    assert (nfix, nlost, len(free)) == (1, 198, 199)
    assert free[0] == 101                      # fixed indices come first
    assert list(free[1:]) == [a for a in range(A) if a not in (33, 101)]  # lost, ascending


def test_free_space_tail_padding_is_not_free():
    # padding bits past A are neither fixed nor lost (free_space_mt..._interlaced.hpp:68-81)
    S, A = 4, 70
    rows = rows_with(S, A, [(i, 5) for i in range(S)])
    free, nfix, nlost = oracle.free_space(rows, A)
    assert nfix == 1 and nlost == A - 1 and max(free) < A


def test_free_space_threads_agree():
    rng = np.random.default_rng(3)
    rows = rng.integers(0, 2 ** 63, size=(33, 24), dtype=np.uint64) & rng.integers(0, 2 ** 63, size=(33, 24),
                                                                                  dtype=np.uint64)
    rows[:, 7] |= np.uint64(0xF0F0)
    a = oracle.free_space(rows, 24 * 64 - 5, threads=1)
    b = oracle.free_space(rows, 24 * 64 - 5, threads=5)
    assert np.array_equal(a[0], b[0]) and a[1:] == b[1:]


# ---- crossover_test.cpp:37-111.  Parent individual 1 = genomes 2 {22, 77, 99}
# and 3 {77, 88, 15}; positions 88->0.75, 99->0.85, 22->0.5622, 15->0.562273;
# one breakpoint at 0.562272.  Before the breakpoint the first strand, after it
# the second: offspring carries 77, 88, 22, 15 and not 99 or 33.
POS = {88: 0.75, 99: 0.85, 22: 0.5622, 15: 0.562273}
EVENT = 0.562272


def crossover_positions(A=150):
    p = np.full(A, 0.999)
    for a, v in POS.items():
        p[a] = v
    return p


def test_block_crossover_fixture():
    pos = crossover_positions()
    r = rows_with(4, 150, [(0, 28), (0, 110), (1, 28), (2, 22), (2, 77), (2, 99), (3, 77), (3, 88), (3, 15)])
    top, bottom = r[2], r[3]
    out = [oracle.block_crossover(int(top[w]), int(bottom[w]), 64 * w, pos, [EVENT]) for w in range(3)]
    child = np.array(out, np.uint64)[None, :]
    for a, want in ((77, True), (33, False), (88, True), (99, False), (22, True), (15, True)):
        assert bit(child, 0, a) == want, a


FIXTURE_BITS = [(0, 28), (0, 110), (1, 28), (2, 22), (2, 77), (2, 99), (3, 77), (3, 88), (3, 15)]


def crossover_engine_case(q1):
    """The crossover fixture through the whole generation step.  Parents: the
    fixture's two individuals; the event list carries the one breakpoint.
    With the reference's quirk (q1) the second gamete of a pair never
    recombines (batch_crossover_taskwe_population_space_row.hpp:133-138), so
    the pair is (parent 1, parent 0) with the breakpoint on gamete 0; without
    it the fixture's own layout (parent 0, parent 1; breakpoint on gamete 1)
    is used.  Returns (start, tape, offspring row that carries the recombinant)."""
    N, A = 2, 150
    rows = rows_with(2 * N, A, FIXTURE_BITS)
    pos = crossover_positions(A)
    if q1:
        pairs, ev_off, kid = np.array([1, 0, 1, 0], np.uint32), np.array([0, 1, 1, 1, 1], np.uint32), 0
    else:
        pairs, ev_off, kid = np.array([0, 1, 0, 1], np.uint32), np.array([0, 0, 1, 1, 1], np.uint32), 1
    tape = oracle.Tape(N, 0, pairs, np.zeros(2 * N, np.uint8), ev_off, np.array([EVENT]), np.zeros(0, np.uint32),
                       np.zeros(0), np.zeros(0, np.float32))
    return (N, rows, pos, np.zeros(A, np.float32)), tape, kid


@pytest.mark.parametrize("q1", [True, False])
def test_crossover_fixture_through_engine(q1):
    (N, rows, pos, eff), tape, kid = crossover_engine_case(q1)
    orc = oracle.Oracle(T=1, mu=0.0, rho=0.0, p_neutral=1.0, q1=q1, threads=1)
    orc.load_population(N, rows, pos, eff)
    orc.step_tape(tape)
    child = orc.rows()
    for a, want in ((77, True), (33, False), (88, True), (99, False), (22, True), (15, True)):
        assert bit(child, kid, a) == want, a
    # the other gamete of the pair comes from parent 0 with no events: genome 0
    other = 1 - kid
    assert bit(child, other, 28) and bit(child, other, 110)


def test_crossover_tie_counts_breakpoint_at_position():
    # upper_bound semantics (classifiers/region_classifier.hpp:73): a breakpoint
    # equal to an allele's position is <= it, so the allele comes from the bottom.
    pos = np.array([0.5, 0.25])
    top, bottom = 0b01, 0b10   # slot 0 on top, slot 1 on bottom
    out = oracle.block_crossover(top, bottom, 0, pos, [0.5])
    # slot 0 (pos 0.5): one breakpoint <= 0.5 -> bottom strand, which lacks it;
    # slot 1 (pos 0.25): none <= 0.25 -> top strand, which lacks it
    assert out == 0
    # moving the breakpoint just above 0.5 keeps slot 0 on the top strand
    assert oracle.block_crossover(top, bottom, 0, pos, [np.nextafter(0.5, 1.0)]) == 0b01


# ---- linear_phenotype_test.cpp:47-137: individual 10 with six (genome, allele)
# pairs; phenotype = sum of the alleles' weights.
def test_linear_phenotype_fixture():
    A, T = 200, 1
    pairs = [(20, 12), (20, 35), (20, 120), (21, 50), (21, 150), (21, 199)]
    rng = np.random.default_rng(1234)
    w = rng.standard_normal(A)
    rows = rows_with(22, A, pairs)
    g20 = oracle.genome_weights(rows[20], w, T)[0]
    g21 = oracle.genome_weights(rows[21], w, T)[0]
    assert g20 == pytest.approx(w[12] + w[35] + w[120], rel=1e-15)
    assert g21 == pytest.approx(w[50] + w[150] + w[199], rel=1e-15)
    assert g20 + g21 == pytest.approx(sum(w[a] for _, a in pairs), rel=1e-15)
    # dyadic weights: every summation order gives the same double
    wd = np.round(w * 1024) / 1024
    exact = sum(wd[a] for _, a in pairs)
    assert oracle.genome_weights(rows[20], wd, T)[0] + oracle.genome_weights(rows[21], wd, T)[0] == exact


def test_phenotype_summation_order_words_up_bits_down():
    # accumulate_allele_weights_alt2: words ascending, bits descending
    # (batch_phenotype_task_population_space_row.hpp:144-149)
    A = 128
    w = np.zeros(A)
    w[0], w[1], w[64] = 1e16, 1.0, -1e16
    row = rows_with(1, A, [(0, 0), (0, 1), (0, 64)])[0]
    got = oracle.genome_weights(row, w, 1)[0]
    want = ((0.0 + w[1]) + w[0]) + w[64]
    assert got == want


# ---- mutation_test.cpp:42-75: 15 mutations into an empty 200-allele space
# leave 185 free slots.
def test_mutation_free_count_fixture():
    N, A = 10, 200
    orc = oracle.Oracle(T=1, mu=0.0, rho=0.0, p_neutral=1.0, threads=1)
    orc.seed_population(N, np.linspace(0, 0.99, A), np.zeros(A, np.float32), np.zeros(A, np.uint32), 1)
    assert orc.info()["A"] == A
    rng = np.random.default_rng(1234)
    M = 15
    t = oracle.Tape(N, M, rng.integers(0, N, 2 * N).astype(np.uint32), np.zeros(2 * N, np.uint8),
                    np.zeros(2 * N + 1, np.uint32), np.zeros(0), rng.integers(0, 2 * N, M).astype(np.uint32),
                    rng.random(M), np.zeros(M, np.float32))
    orc.step_tape(t)
    free, nfix, nlost = oracle.free_space(orc.rows(), A)
    assert len(free) == A - M and nfix == 0


# ---- debruijn_bit_walker_test.cpp / popcount_test.cpp
@pytest.mark.parametrize("w", [0x13, 0x1000F33210220307, 1, 1 << 63, 0])
def test_bit_walker_visits_every_set_bit_once(w):
    idx = oracle.bit_walk(w)
    assert idx == sorted(idx)
    assert sum(1 << i for i in idx) == w
    assert len(idx) == bin(w).count("1")


def test_popcount_known_answers():
    assert bin(0xFFFFFF7F).count("1") == 31
    assert len(oracle.bit_walk(0xCD)) == 5
    assert len(oracle.bit_walk(0xFFFFFF7F00000000)) == 31
    assert len(oracle.bit_walk(0xFFFFFFFF)) == 32


def test_seed_hash_rule():
    # the pre-seeded start shares one integer rule between the oracle and the device
    def splitmix(seed, row, slot):
        m = (1 << 64) - 1
        x = (seed + 0x9E3779B97F4A7C15 * ((row << 32) + slot + 1)) & m
        x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & m
        x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & m
        x ^= x >> 31
        return x >> 32
    for (s, r, a) in [(0, 0, 0), (99, 7, 12345), (2 ** 63 + 5, 4000000, 65535)]:
        assert oracle.seed_hash(s, r, a) == splitmix(s, r, a)
