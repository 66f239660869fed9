"""The oracle against an independent numpy restatement of one generation of
`Engine::simulate` (examples/QTLSim/engine_batched_task.hpp:163-223), on random
populations and random tapes: free space over the parent rows
(free_space_details.hpp:300-357: fixed slots ascending, then lost slots
ascending), fixed-column clearing (engine_batched_task.hpp:303-345), the
child width (:287-301), crossover by breakpoint parity with upper_bound ties
(position_classifier.hpp:59-93, block_crossover.hpp:46-63; Q1 keeps the second
gamete whole), mutation into free slots then appended ones
(batch_mutation_mt.hpp:114-150), per-genome effect sums
(batch_phenotype_mt_population_space_row.hpp:111-156), and the fitness
metrics on the resulting phenotypes (general_fitness.hpp:101-119).  The numpy version
works on whole bit matrices, so it shares no code or loop structure with the
C++ restatement it checks."""
import numpy as np
import pytest

import oracle


def ref_width(A):
    return max(1, -(-A // 512)) * 8


def unpack(rows):
    return np.unpackbits(rows.view(np.uint8).reshape(rows.shape[0], -1), axis=1, bitorder="little").astype(bool)


def pack(bits):
    return np.packbits(bits.astype(np.uint8), axis=1, bitorder="little").view(np.uint64)


def numpy_step(rows, pos, eff, tape, q1):
    """One generation from parent rows (2Np x W) and allele tables; returns child rows, free list,
    allele positions and effects, fixed slots and individual phenotypes."""
    A, T = len(pos), eff.shape[1]
    bits = unpack(rows)
    F, V = bits[:, :A].all(axis=0), bits[:, :A].any(axis=0)
    fixed, lost = np.flatnonzero(F), np.flatnonzero(~V)
    free = np.concatenate([fixed, lost]).astype(np.uint32)
    bits[:, fixed] = False
    M = tape.M
    A2 = A if len(free) >= M else A + (M - len(free))
    W2 = ref_width(A2)
    N = tape.N
    child = np.zeros((2 * N, 64 * W2), bool)
    for g in range(2 * N):
        p, s = int(tape.pairs[g]), int(tape.swap[g])
        top, bot = bits[2 * p + s, :A], bits[2 * p + 1 - s, :A]
        ev = np.sort(tape.ev_pos[tape.ev_off[g]:tape.ev_off[g + 1]])
        if q1 and g % 2 == 1:
            ev = ev[:0]
        switched = (np.searchsorted(ev, pos, side="right") & 1).astype(bool)  # breakpoints <= position
        child[g, :A] = np.where(switched, bot, top)
    slots = np.concatenate([free, np.arange(A, A2, dtype=np.uint32)])[:M]
    pos2 = np.concatenate([pos, np.zeros(A2 - A)])
    eff2 = np.concatenate([eff, np.zeros((A2 - A, T))])
    for i in range(M):
        a = int(slots[i])
        child[tape.mut_seq[i], a] ^= True
        pos2[a] = tape.mut_pos[i]
        eff2[a] = tape.mut_eff[i * T:(i + 1) * T]
    z = child[:, :A2].astype(np.float64) @ eff2
    return pack(child), free, pos2, eff2, fixed, z[0::2] + z[1::2]


def random_case(rng, Np, N, A, T, M, rho):
    W = ref_width(A)
    bits = np.zeros((2 * Np, 64 * W), bool)
    bits[:, :A] = rng.random((2 * Np, A)) < rng.uniform(0.05, 0.6, A)
    bits[:, rng.choice(A, 7, replace=False)] = True           # fixed in the parent population
    bits[:, rng.choice(A, 9, replace=False)] = False          # lost
    pos = rng.random(A)
    pos[:4] = pos[4:8]                                        # shared positions
    eff = rng.standard_normal((A, T)) * (rng.random((A, 1)) < 0.8)
    E = rng.poisson(rho, 2 * N)
    ev_off = np.concatenate([[0], np.cumsum(E)]).astype(np.uint32)
    ev_pos = rng.random(int(E.sum()))
    if len(ev_pos) > 3:
        ev_pos[:3] = pos[rng.choice(A, 3)]                    # breakpoints exactly at allele positions
    tape = oracle.Tape(N, M, rng.integers(0, Np, 2 * N), rng.integers(0, 2, 2 * N), ev_off, ev_pos,
                       rng.integers(0, 2 * N, M), rng.random(M), rng.standard_normal(M * T).astype(np.float32))
    return pack(bits), pos, eff.astype(np.float32), tape


@pytest.mark.parametrize("q1", [True, False])
@pytest.mark.parametrize("Np,N,M", [(30, 30, 5), (30, 12, 60), (12, 40, 20), (25, 25, 0)])
def test_oracle_step_matches_numpy_restatement(q1, Np, N, M):
    rng = np.random.default_rng(1000 * Np + 10 * N + M + q1)
    A, T = 300, 2
    rows, pos, eff, tape = random_case(rng, Np, N, A, T, M, rho=2.5)
    orc = oracle.Oracle(T=T, fitness=oracle.FIT_GAUSSIAN_VS, fit_param=4.0, mu=0.1, rho=2.5, p_neutral=0.0,
                        q1=q1, threads=2, seed=5)
    orc.load_population(Np, rows, pos, eff)
    orc.step_tape(tape)
    want_rows, want_free, want_pos, want_eff, want_fixed, want_z = numpy_step(rows, pos, eff.astype(np.float64),
                                                                              tape, q1)
    got = orc.rows()
    assert got.shape == want_rows.shape
    assert np.array_equal(got, want_rows)
    assert np.array_equal(orc.free_list(), want_free)
    opos, _, oeff = orc.alleles()
    assert np.array_equal(opos, want_pos)
    assert np.array_equal(oeff.reshape(-1, T), want_eff.astype(np.float32).astype(np.float64))
    assert np.array_equal(orc.fixed()[0], pos[want_fixed])
    np.testing.assert_allclose(orc.phenotypes().reshape(-1, T), want_z, rtol=1e-12, atol=1e-12)


def numpy_fitness(z, kind, fit_param, N, mu):
    """The toolkit metrics (normal_fitness_metric.cpp:25-31 with sigma = sqrt(4 N mu), normal_fitness_generator.cpp:36-52;
    quadratic_fitness_metric.cpp:23-28; constant) on trait 0, and exp(-|z|^2 / 2 Vs) over all traits."""
    n4 = np.sqrt(4.0 * N * mu)
    if kind == oracle.FIT_GAUSSIAN:
        return np.exp(-z[:, 0] ** 2 / (2.0 * n4 * n4)) / (n4 * np.sqrt(2.0 * np.pi))
    if kind == oracle.FIT_QUADRATIC:
        r = (z[:, 0] / (fit_param * n4)) ** 2
        return np.where(r >= 1.0, 0.0, 1.0 - r)
    if kind == oracle.FIT_GAUSSIAN_VS:
        return np.exp(-(z ** 2).sum(axis=1) / (2.0 * fit_param))
    return np.ones(len(z))


@pytest.mark.parametrize("kind", [oracle.FIT_GAUSSIAN, oracle.FIT_QUADRATIC, oracle.FIT_GAUSSIAN_VS,
                                  oracle.FIT_CONSTANT])
def test_oracle_fitness_matches_the_metric_formulas(kind):
    rng = np.random.default_rng(77 + kind)
    Np, N, A, T, mu = 30, 24, 300, 2, 0.05
    rows, pos, eff, tape = random_case(rng, Np, N, A, T, 10, rho=1.0)
    # the metric's scale from the phenotypes (numpy restatement), so that its values spread out
    z = numpy_step(rows, pos, eff.astype(np.float64), tape, True)[5]
    n4 = np.sqrt(4.0 * N * mu)
    fit_param = {oracle.FIT_QUADRATIC: float(np.median(np.abs(z[:, 0]))) / n4,
                 oracle.FIT_GAUSSIAN_VS: float(np.median((z ** 2).sum(axis=1))) / 2.0}.get(kind, 1.0)
    orc = oracle.Oracle(T=T, fitness=kind, fit_param=fit_param, mu=mu, rho=1.0, p_neutral=0.0, q1=True,
                        threads=2, seed=5)
    orc.load_population(Np, rows, pos, eff)
    orc.step_tape(tape)
    z = orc.phenotypes().reshape(-1, T)
    f = numpy_fitness(z, kind, fit_param, N, mu)
    if kind == oracle.FIT_QUADRATIC:
        assert 0 < (f == 0.0).sum() < N        # both branches of the metric are exercised
    np.testing.assert_allclose(orc.fitness(), f, rtol=1e-13, atol=1e-300)


def test_oracle_results_do_not_depend_on_its_thread_count():
    # the partitioned stages (crossover by pairs, phenotype by genomes, free space by columns) give the same
    # rows, tables, phenotypes and fitness on one thread and on four, generation after generation
    runs = []
    for threads in (1, 4):
        orc = oracle.Oracle(T=2, fitness=oracle.FIT_GAUSSIAN_VS, fit_param=4.0, mu=0.4, rho=2.0, p_neutral=0.3,
                            q1=False, threads=threads, seed=17)
        orc.init(150)
        states = []
        for N in (150, 150, 90, 200, 200, 60):
            orc.step_record(N)
            states.append((orc.rows(), orc.free_list(), orc.alleles()[0], orc.phenotypes(), orc.fitness()))
        runs.append(states)
    for g, (a, b) in enumerate(zip(*runs)):
        for x, y in zip(a, b):
            assert np.array_equal(x, y), f"generation {g}"
