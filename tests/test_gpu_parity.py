"""GPU parity against the CPU oracle through the C-ABI.

The oracle (oracle/clotho_oracle.cpp, the restatement of QTLSimMT's
Engine::simulate) draws each generation in the reference's order and records
the tape; libclotho_gpu.so replays the same tape.  Bar:
  * bit-exact for integer/bit work: every offspring row, allele count and row
    width, the free list (fixed ascending then lost ascending), counts, the
    allele table (positions, ages), the fixed-allele table;
  * phenotypes: the GPU carries each genome's sum from its parent row and adds
    the switched alleles' effects as FP32 lane sums reduced across the warp in
    FP32 and added to the FP64 carried sum; the FP64
    oracle re-sums every set bit.  Each generation contributes at most the error
    of an FP32 sum of n terms of magnitude <= sum|w|, and carried sums inherit
    their ancestors' residue, so the tolerance written here is population-wide:
    |z_gpu - z_fp64| <= (g + 1) * 2^-24 * max_i[(n_i + 1) * sum_i|w|]
    with n_i the set bits and sum_i|w| the absolute effect sum of individual i
    (both genomes), g generations after the last full evaluation;
  * fitness: equal to the metric applied to the GPU phenotype in FP64
    (rtol 1e-12), and within the propagated phenotype bound of the oracle.
"""
import numpy as np
import pytest

import oracle
from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu

if not gpu_available():  # collected on CPU machines, skipped there
    pytest.skip("no CUDA device", allow_module_level=True)

import clotho_gb300 as cg  # noqa: E402

FITS = {"constant": oracle.FIT_CONSTANT, "gaussian": oracle.FIT_GAUSSIAN, "quadratic": oracle.FIT_QUADRATIC,
        "gaussian_vs": oracle.FIT_GAUSSIAN_VS}


def make_pair(N, A_cap, T=1, fitness="constant", fit_param=1.0, mu=0.05, rho=0.5, bias=0.5, p_neutral=1.0,
              q1=True, seed=11, threads=2):
    orc = oracle.Oracle(T=T, fitness=FITS[fitness], fit_param=fit_param, mu=mu, rho=rho, bias=bias,
                        p_neutral=p_neutral, q1=q1, threads=threads, seed=seed)
    gpu = cg.Population(N, A_cap, T, fitness=fitness, fit_param=fit_param, mu=mu, rho=rho, bias=bias,
                        p_neutral=p_neutral, q1=q1, seed=seed, max_events=int(4 * N * rho + 4096),
                        max_mutations=int(4 * N * mu + 4096), max_fixed=1 << 16)
    return orc, gpu


def pheno_bound(rows, eff, gens=0):
    """(g+1)(n+1) 2^-24 sum|w| per individual from the rows and the FP32 effects.
    Only the nonzero words are unpacked, so populations of 1e5 individuals with
    wide rows fit in host memory."""
    S, W = rows.shape
    A, T = eff.shape
    absw = np.abs(eff.astype(np.float64))
    s = np.zeros((S, T))
    n = np.zeros(S)
    for r0 in range(0, S, 16384):
        r, w = np.nonzero(rows[r0:r0 + 16384])
        if r.size == 0:
            continue
        words = np.ascontiguousarray(rows[r0 + r, w])
        bits = np.unpackbits(words.view(np.uint8).reshape(-1, 8), axis=1, bitorder="little")
        k, b = np.nonzero(bits)
        slot = w[k].astype(np.int64) * 64 + b
        ok = slot < A
        row = r0 + r[k][ok]
        np.add.at(s, row, absw[slot[ok]])
        n += np.bincount(row, minlength=S)
    s_ind = s[0::2] + s[1::2]
    n_ind = (n[0::2] + n[1::2])[:, None]
    worst = ((n_ind + 1.0) * s_ind).max(axis=0) if len(s_ind) else np.zeros(s.shape[1])
    return (gens + 1.0) * 2.0 ** -24 * np.broadcast_to(worst, s_ind.shape) + 1e-30


def fitness_of(z, kind, fit_param, N, mu):
    z = z.astype(np.float64)
    if kind == "constant":
        return np.ones(len(z))
    if kind == "gaussian":
        sig = np.sqrt(4.0 * N * mu)
        return (1.0 / sig) * 0.398942280401432677939946059934 * np.exp(-(z[:, 0] ** 2) / (2 * sig * sig))
    if kind == "quadratic":
        s = fit_param * np.sqrt(4.0 * N * mu)
        r = (z[:, 0] / s) ** 2
        return np.where(r >= 1.0, 0.0, 1.0 - r)
    if kind == "gaussian_vs":
        return np.exp(-(z ** 2).sum(axis=1) / (2 * fit_param))
    raise ValueError(kind)


def compare_state(orc, gpu, g, check_pheno=True, kind="constant", fit_param=1.0, mu=0.0):
    oi, gi = orc.info(), gpu.info()
    assert gi["device_error"] == 0, f"gen {g}: device error {gi['device_error']}"
    for k in ("N", "A", "fixed_count", "lost_count", "free_count", "fixed_total", "generation"):
        assert oi[k] == gi[k], f"gen {g}: {k} oracle={oi[k]} gpu={gi[k]}"
    assert oi["B"] == gi["W"], f"gen {g}: width oracle={oi['B']} gpu={gi['W']}"
    ro, rg = orc.rows(), gpu.rows()
    assert ro.shape == rg.shape
    if not np.array_equal(ro, rg):
        bad = np.argwhere(ro != rg)
        r, w = bad[0]
        raise AssertionError(f"gen {g}: {len(bad)} words differ; first row {r} word {w}: "
                             f"oracle {int(ro[r, w]):#x} gpu {int(rg[r, w]):#x}")
    assert np.array_equal(orc.free_list(), gpu.free_list()), f"gen {g}: free list differs"
    po, ao, eo = orc.alleles()
    pg, ag, eg = gpu.alleles()
    assert np.array_equal(po, pg) and np.array_equal(ao, ag), f"gen {g}: allele table differs"
    assert np.array_equal(eo, eg.astype(np.float64)), f"gen {g}: trait table differs"
    fpo, fao, feo = orc.fixed()
    fpg, fag, feg = gpu.fixed()
    assert np.array_equal(fpo, fpg) and np.array_equal(fao, fag) and np.array_equal(feo, feg.astype(np.float64))
    if check_pheno:
        zo, zg = orc.phenotypes(), gpu.phenotypes().astype(np.float64)
        if oi["all_neutral"]:
            assert np.all(zg == 1.0)
        else:
            bound = pheno_bound(rg, eg, max(g, 0) + 1)
            err = np.abs(zo - zg)
            assert np.all(err <= bound), f"gen {g}: phenotype error {err.max()} > bound"
        fg = gpu.fitness()
        np.testing.assert_allclose(fg, fitness_of(gpu.phenotypes(), kind, fit_param, gi["N"], mu), rtol=1e-12,
                                   atol=1e-300)


def run_parity(G, N, A_cap, **kw):
    orc, gpu = make_pair(N, A_cap, **kw)
    orc.init(N)
    gpu.init(N)
    for g in range(G):
        tape = orc.step_record(N)
        gpu.simulate(tape)
        compare_state(orc, gpu, g, kind=kw.get("fitness", "constant"), fit_param=kw.get("fit_param", 1.0),
                      mu=kw.get("mu", 0.05))
    return orc, gpu


def test_neutral_wright_fisher_bit_exact():
    # C1-shaped (neutral, uniform parents), small N so the oracle is instant
    orc, gpu = run_parity(40, 300, 8192, mu=0.2, rho=0.3, p_neutral=1.0)
    assert orc.info()["A"] > 64


def test_qtl_selection_bit_exact_and_phenotype_bound():
    # C2-shaped: single trait, N(0,1) effects, exp(-z^2/2), fitness-proportional parents
    run_parity(30, 250, 8192, T=1, fitness="gaussian_vs", fit_param=1.0, mu=0.2, rho=1.0, p_neutral=0.0)


def test_four_traits_reference_gaussian_q1_off():
    run_parity(20, 200, 8192, T=4, fitness="gaussian", mu=0.3, rho=3.0, p_neutral=0.3, q1=False)


def test_quadratic_three_traits():
    run_parity(15, 150, 4096, T=3, fitness="quadratic", fit_param=3.0, mu=0.2, rho=2.0, p_neutral=0.5)


def test_many_events_beyond_register_set():
    # rho large enough that many gametes carry more than 16 breakpoints
    run_parity(8, 100, 4096, mu=0.3, rho=24.0, p_neutral=1.0, q1=False)


@pytest.mark.parametrize("A_cap,rho", [(70_000, 1.0), (500_000, 0.8), (70_000, 3.0), (600_000, 1.0)])
def test_wide_allele_space_classifiers(A_cap, rho):
    # capacities above 65,536 slots: up to 524,288 slots and rho <= 1 the suffix table's masks are built
    # chunk by chunk (chunk-mask build); otherwise the interval classifier tests every heterozygous bit by
    # its rank
    run_parity(6, 60, A_cap, T=2, fitness="gaussian_vs", fit_param=4.0, mu=0.5, rho=rho, p_neutral=0.5)


def test_chunk_masks_with_many_breakpoints():
    # the chunk-mask build (70,000 slots; the population's rho of 1 selects it) on tapes drawn with rho = 20
    # and Q1 off: rows of up to 16 breakpoints take their masks from the table, longer ones compare every
    # heterozygous bit with the breakpoint positions
    N, G = 80, 8
    orc = oracle.Oracle(T=2, fitness=FITS["gaussian_vs"], fit_param=4.0, mu=2.0, rho=20.0, p_neutral=0.5,
                        q1=False, threads=2, seed=11)
    gpu = cg.Population(N, 70_000, 2, fitness="gaussian_vs", fit_param=4.0, mu=2.0, rho=1.0, p_neutral=0.5,
                        q1=False, seed=11, max_events=int(4 * N * 20.0 + 4096), max_mutations=int(4 * N * 2.0 + 4096),
                        max_fixed=1 << 16)
    orc.init(N)
    gpu.init(N)
    for g in range(G):
        tape = orc.step_record(N)
        assert np.diff(tape.ev_off).max() > 16
        gpu.simulate(tape)
        compare_state(orc, gpu, g, kind="gaussian_vs", fit_param=4.0, mu=2.0)


def test_suffix_table_boundaries():
    # many alleles with shared positions and breakpoints on and between the
    # 64-rank table rows: corrections from both sides, ties broken by slot
    run_parity(12, 120, 8192, mu=2.0, rho=12.0, p_neutral=1.0, q1=False)


@pytest.mark.parametrize("A_cap,rho", [(4096, 1.5), (70_000, 1.0), (70_000, 1.5)])
def test_staged_policies_equal_fused(A_cap, rho):
    # the staged stage-by-stage calls against the fused step, for each generation-kernel build: bitmap
    # masks, chunk masks (70,000 slots at rho <= 1), interval classifier
    orc, gpu = make_pair(180, A_cap, T=2, fitness="gaussian_vs", fit_param=4.0, mu=0.2, rho=rho, p_neutral=0.4)
    gpu2 = cg.Population(180, A_cap, 2, fitness="gaussian_vs", fit_param=4.0, mu=0.2, rho=rho, p_neutral=0.4,
                         max_events=8192, max_mutations=8192, max_fixed=1 << 16)
    orc.init(180)
    gpu.init(180)
    gpu2.init(180)
    for g in range(12):
        tape = orc.step_record(180)
        gpu.simulate(tape)
        gpu2.simulate_staged(tape)
        compare_state(orc, gpu2, g, kind="gaussian_vs", fit_param=4.0)
        assert np.array_equal(gpu.rows(), gpu2.rows())
        # fused = carried sums, staged = full re-sum: equal within the same bound
        bound = pheno_bound(gpu.rows(), gpu.alleles()[2], g + 1)
        assert np.all(np.abs(gpu.phenotypes() - gpu2.phenotypes()) <= 2 * bound)


def test_seeded_population_parity():
    rng = np.random.default_rng(5)
    N, A, T = 200, 1500, 2
    pos = rng.random(A)
    eff = rng.standard_normal(A * T).astype(np.float32) * 0.1
    thr = (rng.random(A) * 2 ** 32 * 0.3).astype(np.uint32)
    orc, gpu = make_pair(N, 4096, T=T, fitness="gaussian_vs", fit_param=50.0, mu=0.1, rho=2.0, p_neutral=0.2)
    orc.seed_population(N, pos, eff, thr, 99)
    gpu.seed_population(N, pos, eff, thr, 99)
    compare_state(orc, gpu, -1, kind="gaussian_vs", fit_param=50.0)
    for g in range(10):
        gpu.simulate(orc.step_record(N))
        compare_state(orc, gpu, g, kind="gaussian_vs", fit_param=50.0)


@pytest.mark.parametrize("rho", [1.0, 3.0])
def test_rows_wider_than_the_shared_accumulators(rho):
    # 460,000 seeded allele slots (7,192-word rows): wider than the shared-memory AND/OR accumulators of the
    # chunk-mask build (rho = 1: 3,072 words) and of the interval classifier (rho = 3: 6,976 words) hold, so
    # the fold goes to the population's global accumulators and the fixed mask is read from global memory;
    # carrier fractions U[0, 1) give fixed and lost columns, and 4,000 new alleles a generation reuse slots
    rng = np.random.default_rng(17)
    N, A, T = 40, 460_000, 1
    pos = rng.random(A)
    eff = (rng.standard_normal(A * T) * 0.02).astype(np.float32)
    thr = (rng.random(A) * 2 ** 32).astype(np.uint64).clip(0, 2 ** 32 - 1).astype(np.uint32)
    orc, gpu = make_pair(N, 480_000, T=T, fitness="gaussian_vs", fit_param=500.0, mu=50.0, rho=rho,
                         p_neutral=0.3)
    orc.seed_population(N, pos, eff, thr, 7)
    gpu.seed_population(N, pos, eff, thr, 7)
    assert gpu.info()["W"] == 7192
    compare_state(orc, gpu, -1, kind="gaussian_vs", fit_param=500.0)
    for g in range(4):
        gpu.simulate(orc.step_record(N))
        compare_state(orc, gpu, g, kind="gaussian_vs", fit_param=500.0, mu=50.0)
    assert gpu.info()["fixed_total"] > 0 and gpu.info()["W"] > 6976


def test_edge_tie_breakpoint_equals_position():
    # A breakpoint exactly at an allele's position counts as <= (upper_bound,
    # classifiers/region_classifier.hpp:73): that allele comes from the bottom strand.
    N = 4
    orc, gpu = make_pair(N, 1024, mu=0.0, rho=0.0)
    orc.init(N)
    gpu.init(N)
    # generation 1: give every row 3 alleles through mutations, positions 0.25/0.5/0.75
    S = 2 * N
    seq = np.array([0, 1, 1, 2, 3, 4, 5, 6, 7], np.uint32)
    pos = np.array([0.25, 0.5, 0.75, 0.25, 0.5, 0.75, 0.5, 0.25, 0.75])
    t1 = oracle.Tape(N, len(seq), np.arange(S, dtype=np.uint32) // 2 % N, np.zeros(S, np.uint8),
                     np.zeros(S + 1, np.uint32), np.zeros(0), seq, pos, np.zeros(len(seq), np.float32))
    orc.step_tape(t1)
    gpu.simulate(t1)
    compare_state(orc, gpu, 0)
    # generation 2: one breakpoint exactly at 0.5 on every even gamete, swaps alternate
    ev_off = np.zeros(S + 1, np.uint32)
    ev_off[1:] = np.cumsum(np.array([1, 0] * N, np.uint32))
    ev_pos = np.full(N, 0.5)
    pairs = np.array([0, 1, 2, 3, 1, 0, 3, 2], np.uint32)
    t2 = oracle.Tape(N, 0, pairs, np.array([0, 1] * N, np.uint8), ev_off, ev_pos, np.zeros(0, np.uint32),
                     np.zeros(0), np.zeros(0, np.float32))
    orc.step_tape(t2)
    gpu.simulate(t2)
    compare_state(orc, gpu, 1)


def test_edge_append_path_and_fixed_clearing():
    # M > free forces appended slots; a mutation carried by every row becomes
    # fixed, is cleared and recorded, and its slot is reused first.
    N = 3
    S = 2 * N
    orc, gpu = make_pair(N, 2048, mu=0.0, rho=0.0)
    orc.init(N)
    gpu.init(N)
    seq = np.arange(S, dtype=np.uint32)
    t1 = oracle.Tape(N, S, np.zeros(S, np.uint32), np.zeros(S, np.uint8), np.zeros(S + 1, np.uint32), np.zeros(0),
                     seq, np.linspace(0.1, 0.9, S), np.arange(S, dtype=np.float32))
    orc.step_tape(t1)
    gpu.simulate(t1)
    compare_state(orc, gpu, 0)
    # every gamete copies row 0 of parent 0 (slot 0 then present in all rows -> fixed next time)
    t2 = oracle.Tape(N, 700, np.zeros(S, np.uint32), np.zeros(S, np.uint8), np.zeros(S + 1, np.uint32),
                     np.zeros(0), np.arange(700, dtype=np.uint32) % S, np.linspace(0.01, 0.99, 700),
                     np.ones(700, np.float32))
    orc.step_tape(t2)
    gpu.simulate(t2)
    compare_state(orc, gpu, 1)
    t3 = oracle.Tape(N, 5, np.array([0, 1, 2, 0, 1, 2], np.uint32), np.array([0, 1, 0, 1, 0, 1], np.uint8),
                     np.zeros(S + 1, np.uint32), np.zeros(0), np.array([0, 1, 2, 3, 4], np.uint32),
                     np.array([0.3, 0.31, 0.32, 0.33, 0.34]), np.ones(5, np.float32))
    orc.step_tape(t3)
    gpu.simulate(t3)
    compare_state(orc, gpu, 2)
    assert orc.info()["fixed_total"] >= 1


def test_philox_mode_runs_and_is_deterministic():
    kw = dict(fitness="gaussian_vs", fit_param=2.0, mu=0.1, rho=1.0, p_neutral=0.5, seed=2024,
              max_events=1 << 16, max_mutations=1 << 14, max_fixed=1 << 16)
    a = cg.Population(2000, 1 << 14, 2, **kw)
    b = cg.Population(2000, 1 << 14, 2, **kw)
    a.init(2000)
    b.init(2000)
    a.run_philox(2000, 30)
    for _ in range(30):
        b.simulate_philox(2000)
    a.check()
    assert np.array_equal(a.rows(), b.rows())
    assert np.array_equal(a.phenotypes(), b.phenotypes())
    assert a.info()["A"] > 100


@pytest.mark.parametrize("q1", [True, False])
def test_crossover_fixture_on_gpu(q1):
    # unittest/data_spaces/crossover_test.cpp:37-111 restated (tests/test_oracle_kat.py)
    from tests.test_oracle_kat import crossover_engine_case, bit
    (N, rows, pos, eff), tape, kid = crossover_engine_case(q1)
    orc = oracle.Oracle(T=1, mu=0.0, rho=0.0, p_neutral=1.0, q1=q1, threads=1)
    gpu = cg.Population(N, 150, 1, mu=0.0, rho=0.0, p_neutral=1.0, q1=q1, max_events=16, max_mutations=16)
    orc.load_population(N, rows, pos, eff)
    gpu.load_population(N, rows, pos, eff)
    assert np.array_equal(gpu.rows(), orc.rows())
    orc.step_tape(tape)
    gpu.simulate(tape)
    child = gpu.rows()
    assert np.array_equal(child, orc.rows())
    for a, want in ((77, True), (33, False), (88, True), (99, False), (22, True), (15, True)):
        assert bit(child, kid, a) == want, a


def test_c2_shaped_phenotype_error_stays_within_fp32_bound(capsys):
    # QTL + selection shape: T=1, N(0,1) effects on every new allele, exp(-z^2/2),
    # fitness-proportional parents; 100 generations of carried FP32 sums against
    # the oracle's FP64 re-sums.  Prints the max / mean absolute error.
    N, G = 1000, 100
    orc, gpu = make_pair(N, 1 << 14, T=1, fitness="gaussian_vs", fit_param=1.0, mu=0.1, rho=1.0, p_neutral=0.0)
    orc.init(N)
    gpu.init(N)
    worst, means, scale = 0.0, [], 0.0
    for g in range(G):
        gpu.simulate(orc.step_record(N))
        zo, zg = orc.phenotypes(), gpu.phenotypes()
        err = np.abs(zo - zg)
        bound = pheno_bound(gpu.rows(), gpu.alleles()[2], g + 1)
        assert np.all(err <= bound), f"gen {g}: {err.max()} > bound"
        worst = max(worst, float(err.max()))
        means.append(float(err.mean()))
        scale = max(scale, float(np.abs(zo).max()))
    assert np.array_equal(orc.rows(), gpu.rows())
    with capsys.disabled():
        print(f"\nC2-shaped N={N} G={G}: phenotype |FP32 carried - FP64| max {worst:.3e}, mean {np.mean(means):.3e}"
              f" (|z| up to {scale:.2f}, alleles {gpu.info()['A']})")


@pytest.mark.parametrize("q1", [True, False])
def test_narrow_rows_many_breakpoints(q1):
    # 512 slots (8-word rows): the narrow build of the kernel (copy rows by direct loads) and the one-pass
    # mask build (every breakpoint's table words loaded at once), with up to 32 breakpoints a gamete and
    # the rare longer lists on the per-table-row path; new alleles and phenotypes through the plan
    run_parity(10, 100, 512, T=2, fitness="gaussian_vs", fit_param=4.0, mu=0.1, rho=20.0, p_neutral=0.3, q1=q1)


@pytest.mark.parametrize("A_cap", [8192, 16384])
def test_long_run_stays_bit_exact(A_cap):
    # hundreds of generations: alleles fix and are cleared, slots are recycled through the free list, the
    # fixed table grows and the row width changes; every generation is compared (8,192 slots run the
    # narrow build of the generation kernel, 16,384 the wide one)
    orc, gpu = run_parity(1000, 150, A_cap, T=2, fitness="gaussian_vs", fit_param=8.0, mu=0.1, rho=2.0,
                          p_neutral=0.5)
    i = orc.info()
    assert i["fixed_total"] > 0 and i["generation"] > 1000


@pytest.mark.parametrize("q1", [True, False])
def test_seeded_wide_rows_bench_shape(q1):
    # the N=1e6 bench workload's shape at small N: 50,000 seeded alleles in 65,536 slots (about 780-word rows,
    # the wide build: bulk-copied copy rows, masks from one suffix-table row at a time, large effect gathers
    # in both directions), four traits, rho = 5, the reference gaussian metric
    rng = np.random.default_rng(17)
    N, A, T = 150, 50_000, 4
    pos = rng.random(A)
    eff = rng.standard_normal(A * T).astype(np.float32)
    k = np.minimum(np.floor(1.0 / rng.random(A)), 2 * N - 1)          # carrier counts ~ 1/i
    thr = np.minimum(k / (2 * N) * 2.0 ** 32, 2.0 ** 32 - 1).astype(np.uint32)
    orc, gpu = make_pair(N, 65_536, T=T, fitness="gaussian", mu=0.01, rho=5.0, p_neutral=0.0, q1=q1)
    orc.seed_population(N, pos, eff, thr, 7)
    gpu.seed_population(N, pos, eff, thr, 7)
    compare_state(orc, gpu, -1, kind="gaussian", mu=0.01)
    for g in range(6):
        gpu.simulate(orc.step_record(N))
        compare_state(orc, gpu, g, kind="gaussian", mu=0.01)
    assert gpu.info()["W"] > 512


def test_tape_replay_is_deterministic():
    # the same tapes replayed into two populations give bit-identical phenotypes and fitness, not only
    # genomes: a row with several new alleles adds their FP32 effects in mutation-index order, whatever
    # order the device's counting sort scattered them in (mu = 1.5 puts two or more new alleles on
    # about half of the rows; a few rows get more than 16, the heapsort branch)
    N, G = 300, 25
    orc, a = make_pair(N, 1 << 15, T=4, fitness="gaussian", mu=1.5, rho=1.0, p_neutral=0.0)
    _, b = make_pair(N, 1 << 15, T=4, fitness="gaussian", mu=1.5, rho=1.0, p_neutral=0.0)
    orc.init(N)
    a.init(N)
    b.init(N)
    multi = 0
    for g in range(G):
        tape = orc.step_record(N)
        multi += int((np.bincount(tape.mut_seq, minlength=2 * N) >= 2).sum())
        a.simulate(tape)
        b.simulate(tape)
        assert np.array_equal(a.phenotypes(), b.phenotypes()), f"gen {g}"
        assert np.array_equal(a.fitness(), b.fitness()), f"gen {g}"
    assert np.array_equal(a.rows(), b.rows())
    assert np.array_equal(orc.rows(), a.rows())
    assert a.info()["device_error"] == 0
    assert multi > G * N // 2


def hand_tape(rng, N, T, heavy):
    """A tape with uniform parents, Poisson(0.5) sorted breakpoints per gamete and, besides one new
    allele on every fourth row, `heavy[row]` new alleles on the given rows, all in shuffled order."""
    S = 2 * N
    E = rng.poisson(0.5, S)
    ev_off = np.concatenate([[0], np.cumsum(E)]).astype(np.uint32)
    ev_pos = np.concatenate([np.sort(rng.random(e)) for e in E] + [np.zeros(0)])
    seq = np.concatenate([np.arange(0, S, 4)] + [np.full(n, r) for r, n in heavy.items()])
    seq = rng.permutation(seq).astype(np.uint32)
    M = len(seq)
    return oracle.Tape(N, M, rng.integers(0, N, S), rng.integers(0, 2, S), ev_off, ev_pos, seq, rng.random(M),
                       rng.standard_normal(M * T).astype(np.float32))


def test_tape_rows_with_many_new_alleles_sort_their_lists():
    # hand-made tapes sending 40 new alleles to one row and 17 to another (past the insertion-sort bound,
    # so the heapsort branch orders them) and 3 to a third, in shuffled order: genomes match the oracle
    # bit for bit, phenotypes stay within the FP32 bound, and two replays agree bit for bit
    N, T = 64, 2
    rng = np.random.default_rng(5)
    orc, a = make_pair(N, 4096, T=T, fitness="constant", mu=0.01, rho=0.5, p_neutral=0.0)
    _, b = make_pair(N, 4096, T=T, fitness="constant", mu=0.01, rho=0.5, p_neutral=0.0)
    orc.init(N)
    a.init(N)
    b.init(N)
    for g in range(4):
        tape = hand_tape(rng, N, T, {5: 40, 90: 17, 33: 3})
        orc.step_tape(tape)
        a.simulate(tape)
        b.simulate(tape)
        assert np.array_equal(orc.rows(), a.rows()), f"gen {g}"
        assert np.array_equal(a.phenotypes(), b.phenotypes()), f"gen {g}"
        err = np.abs(orc.phenotypes() - a.phenotypes())
        assert np.all(err <= pheno_bound(a.rows(), a.alleles()[2], g + 1)), f"gen {g}"
    assert a.info()["device_error"] == 0


@pytest.mark.parametrize("mu", [0.3, 1.0])
@pytest.mark.parametrize("q1", [True, False])
def test_population_size_changing_every_generation(q1, mu):
    # a growth model's sizes through the tape call: the population grows, shrinks to one individual and
    # regrows (row counts, parent ranges and fitness tables change every generation; after the bottleneck
    # almost every allele is lost and the new ones reuse the slots); at mu = 1 the rows also widen from 8
    # to 16 to 24 words in generations that change the size; bit-exact against the oracle throughout
    sizes = [150, 220, 90, 90, 300, 40, 1, 2, 60, 200, 299, 17]
    orc, gpu = make_pair(300, 4096, T=2, fitness="gaussian_vs", fit_param=4.0, mu=mu, rho=1.0, p_neutral=0.3,
                         q1=q1)
    orc.init(sizes[0])
    gpu.init(sizes[0])
    lost, alleles = 0, 1
    for g, N in enumerate(sizes):
        gpu.simulate(orc.step_record(N))
        compare_state(orc, gpu, g, kind="gaussian_vs", fit_param=4.0)
        info = gpu.info()
        assert info["N"] == N
        if N == 2:  # the generation after the single-individual one
            lost, alleles = info["lost_count"], info["A"]
    assert lost > 0.9 * alleles


@pytest.mark.parametrize("bias", [0.0, 1.0, 0.3])
def test_device_draws_copy_the_reported_parent_strand(bias):
    # device-drawn generations without breakpoints or new alleles: every offspring row is a copy of one
    # strand of the parent that pairs() reports for it, the second strand exactly when the strand-swap
    # draw (probability bias) says so; the first step runs on a fresh context (no tape step before it)
    rng = np.random.default_rng(23)
    N, A = 400, 3000
    pos = rng.random(A)
    thr = (rng.random(A) * 0.3 * 2.0 ** 32).astype(np.uint32)  # carried by under 30% of rows: none fixed
    pop = cg.Population(N, 4096, 1, mu=0.0, rho=0.0, bias=bias, p_neutral=1.0, seed=29)
    pop.seed_population(N, pos, np.zeros(A, np.float32), thr, 31)
    swaps, total = 0, 0
    for g in range(3):
        parent = pop.rows()
        pop.simulate_philox(N)
        child, pairs = pop.rows(), pop.pairs()
        assert child.shape == parent.shape and pairs.max() < N
        for r in range(2 * N):
            top, bot = parent[2 * pairs[r]], parent[2 * pairs[r] + 1]
            is_top, is_bot = np.array_equal(child[r], top), np.array_equal(child[r], bot)
            assert is_top or is_bot, f"gen {g} row {r}: not a copy of parent {pairs[r]}"
            if is_top != is_bot:
                swaps += int(is_bot)
                total += 1
    assert pop.info()["device_error"] == 0 and total > 0.95 * 3 * 2 * N
    frac = swaps / total
    if bias in (0.0, 1.0):
        assert frac == bias
    else:
        assert abs(frac - bias) < 5 * np.sqrt(bias * (1 - bias) / total)


def test_device_draws_with_the_size_changing_copy_the_reported_parents():
    # device-drawn copy generations (no breakpoints, no new alleles) while the population shrinks tenfold,
    # grows and shrinks again: each offspring row is one strand of the parent pairs() reports for it, less
    # the alleles every parent row carries (fixed: cleared before the copy; after the one-individual
    # generation these are the alleles on both of its strands)
    rng = np.random.default_rng(41)
    N0, A = 400, 2000
    pos = rng.random(A)
    thr = (rng.random(A) * 0.3 * 2.0 ** 32).astype(np.uint32)
    pop = cg.Population(N0, 4096, 1, mu=0.0, rho=0.0, bias=0.5, p_neutral=1.0, seed=43)
    pop.seed_population(N0, pos, np.zeros(A, np.float32), thr, 47)
    for g, N in enumerate([40, 400, 7, 300, 1, 90]):
        parent = pop.rows()
        pN = parent.shape[0] // 2
        parent = parent & ~np.bitwise_and.reduce(parent, axis=0)
        pop.simulate_philox(N)
        child, pairs = pop.rows(), pop.pairs()
        assert child.shape[0] == 2 * N and len(pairs) == 2 * N and pairs.max() < pN, f"gen {g}"
        for r in range(2 * N):
            p = int(pairs[r])
            assert np.array_equal(child[r], parent[2 * p]) or np.array_equal(child[r], parent[2 * p + 1]), \
                f"gen {g} (N {pN} -> {N}) row {r}: not a strand of parent {p}"
    assert pop.info()["device_error"] == 0


def test_staged_policies_with_the_size_changing():
    # the stage-by-stage calls on a population that shrinks more than twofold and regrows: the same rows
    # as the fused step and the oracle
    sizes = [180, 60, 200, 25, 180, 90]
    orc, gpu = make_pair(200, 4096, T=2, fitness="gaussian_vs", fit_param=4.0, mu=0.2, rho=1.5, p_neutral=0.4)
    gpu2 = cg.Population(200, 4096, 2, fitness="gaussian_vs", fit_param=4.0, mu=0.2, rho=1.5, p_neutral=0.4,
                         max_events=8192, max_mutations=8192, max_fixed=1 << 16)
    orc.init(sizes[0])
    gpu.init(sizes[0])
    gpu2.init(sizes[0])
    for g, N in enumerate(sizes):
        tape = orc.step_record(N)
        gpu.simulate(tape)
        gpu2.simulate_staged(tape)
        compare_state(orc, gpu2, g, kind="gaussian_vs", fit_param=4.0)
        assert np.array_equal(gpu.rows(), gpu2.rows()), f"gen {g}"


def test_pairs_report_the_parents_of_the_last_generation_on_every_path():
    # tape steps alternate between two upload sets; device-drawn and staged steps use the first one.  After
    # every step, in any order, pairs() returns the parents that step used (the tape's own, for tape steps)
    N = 120
    orc, gpu = make_pair(N, 4096, T=1, mu=0.1, rho=1.0, p_neutral=1.0)
    orc.init(N)
    gpu.init(N)
    for g, kind in enumerate(["tape", "tape", "tape", "philox", "tape", "staged", "tape", "philox", "philox",
                              "staged", "staged", "tape"]):
        if kind == "philox":
            gpu.simulate_philox(N)
            got = gpu.pairs()
            assert len(got) == 2 * N and got.max() < N, f"step {g}"
            # the device-drawn parents explain the rows: continue the oracle from the GPU's state
            orc.load_population(N, gpu.rows(), *gpu.alleles()[0:3:2])
            continue
        tape = orc.step_record(N)
        if kind == "tape":
            gpu.simulate(tape)
        else:
            gpu.simulate_staged(tape)
        assert np.array_equal(gpu.pairs(), tape.pairs), f"step {g} ({kind})"
        assert np.array_equal(gpu.rows(), orc.rows()), f"step {g} ({kind})"


def test_c1_neutral_wright_fisher_at_its_stated_size():
    # the neutral configuration as stated: N = 1e4 diploid (2e4 rows), mu = 0.01 per sequence, rho = 0.01
    # per gamete, uniform parents, 1,000 generations, free-space analysis every generation; every
    # generation's state compared with the oracle
    from clotho_gb300 import workloads
    w = workloads.NEUTRAL_WF
    orc, gpu = make_pair(w.N, w.max_alleles, T=1, fitness="constant", mu=w.mu, rho=w.rho, p_neutral=1.0,
                         seed=20261203, threads=4)
    orc.init(w.N)
    gpu.init(w.N)
    for g in range(w.generations):
        gpu.simulate(orc.step_record(w.N))
        compare_state(orc, gpu, g, kind="constant", mu=w.mu)
    i = gpu.info()
    assert i["generation"] == w.generations + 1 and i["A"] > 1000


def test_c2_qtl_selection_at_its_stated_population_size(capsys):
    # the QTL-with-selection configuration at its stated size: N = 1e5 (2e5 rows), mu = 0.1 per sequence
    # (2e4 new alleles a generation), rho = 1, one trait with N(0,1) effects, exp(-z^2/2), parents from the
    # FP64 prefix sum over 1e5 fitness values (25 scan chunks), parent-major ordering over 1e5 parents; the
    # allele count passes 65,536 slots, so the chunk-mask build runs.  12 generations (the oracle's
    # cost grows with the rows' width); state compared every fourth generation and at the end.
    import os
    from clotho_gb300 import workloads
    w = workloads.QTL_SELECTION
    G = 12
    orc, gpu = make_pair(w.N, w.max_alleles, T=1, fitness="gaussian_vs", fit_param=w.fit_param, mu=w.mu,
                         rho=w.rho, p_neutral=w.p_neutral, seed=4242, threads=os.cpu_count() or 4)
    orc.init(w.N)
    gpu.init(w.N)
    worst, mean = 0.0, 0.0
    for g in range(G):
        gpu.simulate(orc.step_record(w.N))
        if g % 4 == 3 or g == G - 1:
            compare_state(orc, gpu, g, kind="gaussian_vs", fit_param=w.fit_param, mu=w.mu)
            err = np.abs(orc.phenotypes() - gpu.phenotypes())
            worst, mean = max(worst, float(err.max())), float(err.mean())
    i = gpu.info()
    assert i["A"] > 65_536
    with capsys.disabled():
        print(f"\nC2 at N={w.N} G={G}: rows bit-exact; phenotype |FP32 carried - FP64| max {worst:.3e}, "
              f"mean {mean:.3e} at generation {G} (alleles {i['A']}, row width {i['W']} words)")
