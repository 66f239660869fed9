"""Edge cases through the C-ABI: very long breakpoint lists, tapes with
out-of-range indices, overflow of the allele, fixed-allele, event and
mutation capacities, all-zero fitness and a one-individual population.  Invalid tape entries are bounds-checked on the
device: they are skipped and reported as sticky error bits
(CLOTHO_DEVERR_*), and the population stays usable."""
import numpy as np
import pytest

import oracle
from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu

if not gpu_available():  # collected on CPU machines, skipped there
    pytest.skip("no CUDA device", allow_module_level=True)

import clotho_gb300 as cg  # noqa: E402
from tests.test_gpu_parity import compare_state, make_pair  # noqa: E402



def _tape(N, pairs, mut_seq, mut_pos=None, rng=None):
    S = 2 * N
    M = len(mut_seq)
    rng = rng or np.random.default_rng(0)
    return oracle.Tape(N, M, np.asarray(pairs, np.uint32), np.zeros(S, np.uint8), np.zeros(S + 1, np.uint32),
                       np.zeros(0), np.asarray(mut_seq, np.uint32),
                       rng.random(M) if mut_pos is None else mut_pos, np.zeros(M, np.float32))


def test_rows_with_more_than_128_breakpoints_match_the_oracle():
    # rho = 150: most gametes carry more breakpoints than the device draws per
    # gamete (128), so tape rows take the direct event-compare path
    N = 40
    orc, gpu = make_pair(N, 8192, mu=1.0, rho=150.0, p_neutral=1.0, q1=False)
    orc.init(N)
    gpu.init(N)
    for g in range(6):
        tape = orc.step_record(N)
        assert (np.diff(tape.ev_off) > 128).any()
        gpu.simulate(tape)
        compare_state(orc, gpu, g)


def test_out_of_range_tape_indices_are_flagged_and_skipped():
    N = 30
    gpu = cg.Population(N, 4096, 1, mu=0.0, rho=0.0, p_neutral=1.0, max_events=64, max_mutations=64)
    gpu.init(N)
    rng = np.random.default_rng(1)
    gpu.simulate(_tape(N, rng.integers(0, N, 2 * N), [0, 5, 7], rng=rng))   # three alleles
    assert gpu.info()["device_error"] == 0 and gpu.info()["A"] == 3
    pairs = rng.integers(0, N, 2 * N)
    pairs[3] = N + 5                                   # no such parent
    gpu.simulate(_tape(N, pairs, [1, 2 * N + 9], rng=rng))   # second mutation: no such row
    err = gpu.info()["device_error"]
    assert err & 8 and err & 16                        # CLOTHO_DEVERR_PARENT, CLOTHO_DEVERR_SEQ
    with pytest.raises(cg.ClothoError):
        gpu.check()
    rows = gpu.rows()
    assert rows.shape[0] == 2 * N
    gpu.simulate(_tape(N, rng.integers(0, N, 2 * N), [], rng=rng))          # still usable afterwards
    assert gpu.info()["generation"] == 4
    gpu.close()


def test_allele_capacity_overflow_is_flagged_and_capped():
    N = 20
    gpu = cg.Population(N, 4096, 1, mu=0.0, rho=0.0, p_neutral=1.0, max_events=64, max_mutations=8192)
    gpu.init(N)
    rng = np.random.default_rng(2)
    gpu.simulate(_tape(N, rng.integers(0, N, 2 * N), rng.integers(0, 2 * N, 5000), rng=rng))
    i = gpu.info()
    assert i["device_error"] & 1                       # CLOTHO_DEVERR_ALLELES
    assert i["A"] == 4096 and i["W"] == 64
    rows = gpu.rows()
    bits = np.unpackbits(rows.view(np.uint8).reshape(rows.shape[0], -1), axis=1, bitorder="little")
    assert bits.sum() <= 4096                          # mutations past the capacity were dropped
    gpu.simulate(_tape(N, rng.integers(0, N, 2 * N), [], rng=rng))
    assert gpu.info()["A"] <= 4096
    gpu.close()


def test_all_zero_fitness_falls_back_to_uniform_selection():
    # every individual carries large effects; quadratic fitness with a tiny scale is zero for all
    N, A = 100, 40
    gpu = cg.Population(N, 4096, 1, fitness="quadratic", fit_param=1e-3, mu=0.01, rho=0.5, p_neutral=0.0,
                        max_events=4096, max_mutations=1024)
    gpu.seed_population(N, np.linspace(0.01, 0.99, A), np.full(A, 10.0, np.float32),
                        np.full(A, 2 ** 31, np.uint32), 7)   # each allele in about half the rows
    gpu.simulate_philox(N)
    gpu.simulate_philox(N)
    i = gpu.info()
    assert i["device_error"] & 64                      # CLOTHO_DEVERR_FITNESS
    assert i["N"] == N and i["generation"] == 3
    gpu.close()


def test_one_individual_population():
    gpu = cg.Population(1, 4096, 2, fitness="gaussian_vs", fit_param=2.0, mu=0.5, rho=2.0, p_neutral=0.2,
                        max_events=256, max_mutations=256)
    gpu.init(1)
    gpu.run_philox(1, 25)
    gpu.check()
    i = gpu.info()
    assert i["N"] == 1 and gpu.rows().shape[0] == 2
    assert np.isfinite(gpu.phenotypes()).all()
    gpu.close()


def test_fixed_table_overflow_is_flagged_and_capped():
    # every offspring row copies one strand, so the next step finds all of its alleles fixed: more than the
    # fixed table holds.  The first max_fixed are recorded (the oracle's list is unbounded), the rest are
    # still cleared and their slots freed, so rows and free list stay bit-exact
    N, A = 20, 40
    orc = oracle.Oracle(T=1, fitness=oracle.FIT_CONSTANT, mu=0.0, rho=0.0, p_neutral=1.0, q1=True, threads=1, seed=3)
    gpu = cg.Population(N, 4096, 1, mu=0.0, rho=0.0, p_neutral=1.0, max_events=64, max_mutations=64, max_fixed=4)
    pos, eff, thr = np.linspace(0.01, 0.99, A), np.zeros(A, np.float32), np.full(A, 2 ** 31, np.uint32)
    orc.seed_population(N, pos, eff, thr, 7)
    gpu.seed_population(N, pos, eff, thr, 7)
    rng = np.random.default_rng(4)
    for pairs in (np.zeros(2 * N), rng.integers(0, N, 2 * N), rng.integers(0, N, 2 * N)):
        tape = _tape(N, pairs, [], rng=rng)
        orc.step_tape(tape)
        gpu.simulate(tape)
        assert np.array_equal(orc.rows(), gpu.rows())
        assert np.array_equal(orc.free_list(), gpu.free_list())
    i, oi = gpu.info(), orc.info()
    assert oi["fixed_total"] > 4
    assert i["device_error"] & 2                       # CLOTHO_DEVERR_FIXED
    assert i["fixed_total"] == 4
    assert np.array_equal(gpu.fixed()[0], orc.fixed()[0][:4])
    gpu.close()


def test_device_event_overflow_is_flagged_and_clamped():
    # device-drawn breakpoint counts past 128 a gamete are clamped to 128 and flagged; the run goes on
    N = 50
    gpu = cg.Population(N, 4096, 1, mu=0.05, rho=300.0, p_neutral=1.0, max_events=1 << 16, max_mutations=1024)
    gpu.init(N)
    gpu.simulate_philox(N)
    gpu.simulate_philox(N)
    i = gpu.info()
    assert i["device_error"] & 4                       # CLOTHO_DEVERR_EVENTS
    assert i["generation"] == 3 and i["N"] == N
    gpu.close()


def test_device_mutation_overflow_is_flagged_and_capped():
    # a device-drawn mutation count past max_mutations is capped at it and flagged
    N = 100
    gpu = cg.Population(N, 1 << 14, 1, mu=5.0, rho=0.5, p_neutral=1.0, max_events=4096, max_mutations=64)
    gpu.init(N)
    gpu.simulate_philox(N)
    i = gpu.info()
    assert i["device_error"] & 32                      # CLOTHO_DEVERR_MUT
    assert i["last_M"] == 64 and i["A"] <= 64
    gpu.simulate_philox(N)
    assert gpu.info()["generation"] == 3
    gpu.close()


def test_copy_wait_limit_flags_late_copies_and_changes_no_result():
    # copy rows of wide populations (rows above 128 words) receive their parent strand by bulk copy; with a
    # wait limit of one round (a probe that does not wait) every such copy outlives the limit: the STALL
    # bit is raised, the warps keep waiting for their copies, no copy is abandoned, and rows, phenotypes
    # and fitness equal those of the same run with the default limit
    rng = np.random.default_rng(3)
    N, A = 300, 20_000
    pos = rng.random(A)
    eff = rng.standard_normal(A).astype(np.float32)
    thr = (rng.random(A) * 0.2 * 2.0 ** 32).astype(np.uint32)
    kw = dict(fitness="gaussian_vs", fit_param=4.0, mu=0.05, rho=1.0, p_neutral=0.0, seed=5,
              max_events=1 << 14, max_mutations=1 << 12)
    late = cg.Population(N, 32_768, 1, **kw)
    ref = cg.Population(N, 32_768, 1, **kw)
    for p in (late, ref):
        p.seed_population(N, pos, eff, thr, 9)
    assert late.info()["W"] > 128
    late.set_copy_wait_limit(1)
    late.run_philox(N, 4)
    ref.run_philox(N, 4)
    err = late.info()["device_error"]
    assert err & 128, "a one-round limit must flag the copies"
    assert not err & 256, "no copy may be abandoned"
    assert ref.info()["device_error"] == 0
    assert np.array_equal(late.rows(), ref.rows())
    assert np.array_equal(late.phenotypes(), ref.phenotypes())
    assert np.array_equal(late.fitness(), ref.fitness())
    with pytest.raises(cg.ClothoError):
        late.set_copy_wait_limit(1 << 31)
    late.set_copy_wait_limit(0)
