"""Device-drawn generations (Philox on the device, parents from an FP64 prefix
sum of fitness) pinned to the oracle.

This is the mode the N=1e6 measurement runs.  Its draw rules are restated in
numpy (oracle/device_draws.py), and these tests
  * replay the selection stage (SelectionGenerator::update,
    general_fitness_selection_generator.hpp:45-69) parent for parent, through
    the staged call and inside the fused step, at population sizes whose
    prefix sum spans one and many 4,096-entry chunks, including both uniform
    branches (every fitness equal; total fitness zero);
  * test the sampled parents' counts against fitness / total (chi-square)
    under strong selection;
  * rebuild the event tape of device-drawn generations from the restated draws
    and replay it through the oracle: genomes, free lists, allele and fixed
    tables bit-exact, phenotypes within the FP32 bound of tests/test_gpu_parity.py, at small sizes and
    on the N=1e6 measurement workload itself (2e6 rows, two generations; about a minute and 60 GB of host
    memory);
  * compare site-frequency spectra, segregating sites, heterozygosity and mean
    fitness of device-drawn runs with oracle runs of the same parameters that
    draw from the oracle's own generator (the large-population configuration's
    acceptance check: device Philox draws checked by SFS against the event-tape
    oracle; statistics as population_space_row_frequency_evaluator.hpp:37-62).
"""
import math

import numpy as np
import pytest

import oracle
from oracle import device_draws as dd
from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu

if not gpu_available():  # collected on CPU machines, skipped there
    pytest.skip("no CUDA device", allow_module_level=True)

import clotho_gb300 as cg  # noqa: E402
from clotho_gb300 import workloads  # noqa: E402
from tests.test_gpu_parity import FITS, compare_state, fitness_of  # noqa: E402


def random_start(N, A, T, rng, density=0.3, scale=0.3):
    """Rows (2N x ceil(A/512)*8 words), positions and FP32 effects of an explicit start."""
    W = ((A + 511) // 512) * 8
    bits = rng.random((2 * N, W * 64)) < density
    bits[:, A:] = False
    rows = np.packbits(bits, axis=1, bitorder="little").view(np.uint64)
    return rows, rng.random(A), (rng.standard_normal(A * T) * scale).astype(np.float32)


def loaded(N, A, T, fitness, fit_param, seed, rng, cap_N=None, mu=0.01, rho=0.5, **kw):
    pop = cg.Population(cap_N or N, max(A, 1024), T, fitness=fitness, fit_param=fit_param, mu=mu, rho=rho,
                        p_neutral=0.0, seed=seed, max_events=int(4 * (cap_N or N) * rho + 4096),
                        max_mutations=int(4 * (cap_N or N) * mu + 4096), **kw)
    rows, pos, eff = random_start(N, A, T, rng)
    pop.load_population(N, rows, pos, eff)
    return pop


# ---------------------------------------------------------------------------
# selection stage

@pytest.mark.parametrize("N,N2", [(3000, 3000), (10_000, 9_000), (10_000, 12_500), (100_000, 100_000)])
def test_staged_selection_replays_parent_for_parent(N, N2):
    rng = np.random.default_rng(N + N2)
    seed = 0x5EED0000 + N2
    pop = loaded(N, 512, 2, "gaussian_vs", 10.0, seed, rng, cap_N=max(N, N2))
    fit = pop.fitness()
    gen = pop.info()["generation"]
    assert fit.min() < 0.5 * fit.max(), "selection should not be near-uniform here"
    pop.begin_generation(N2, 0)
    got = pop.select(N2)
    exp, uniform, cdf, total = dd.select_parents(fit, N2, gen, seed)
    assert not uniform
    assert np.array_equal(got, exp), f"{int(np.sum(got != exp))} of {got.size} parents differ"
    pop.close()


def test_fused_step_selection_replays_every_generation():
    rng = np.random.default_rng(7)
    N, seed = 6000, 0xC10
    pop = loaded(N, 1024, 4, "gaussian", 1.0, seed, rng, mu=0.02, rho=5.0)
    for g in range(5):
        fit = pop.fitness()
        gen = pop.info()["generation"]
        pop.simulate_philox(N)
        got = pop.pairs()
        exp, uniform, _, _ = dd.select_parents(fit, N, gen, seed)
        assert not uniform
        assert np.array_equal(got, exp), f"step {g}: {int(np.sum(got != exp))} parents differ"
    pop.check()


def test_selection_is_uniform_when_every_fitness_is_equal():
    rng = np.random.default_rng(11)
    N, seed = 5000, 77
    # constant metric
    pop = loaded(N, 512, 1, "constant", 1.0, seed, rng)
    fit, gen = pop.fitness(), pop.info()["generation"]
    pop.simulate_philox(N)
    exp, uniform, _, _ = dd.select_parents(fit, N, gen, seed)
    assert uniform and np.array_equal(pop.pairs(), exp)
    pop.close()
    # a selective metric over identical individuals: equal, non-unit fitness
    pop = cg.Population(N, 1024, 2, fitness="gaussian_vs", fit_param=3.0, mu=0.0, rho=0.0, p_neutral=0.0, seed=seed)
    rows, pos, eff = random_start(1, 512, 2, rng)
    rows = np.tile(rows, (N, 1))
    pop.load_population(N, rows, pos, eff)
    fit, gen = pop.fitness(), pop.info()["generation"]
    assert np.all(fit == fit[0]) and fit[0] < 1.0
    pop.begin_generation(N, 0)
    got = pop.select(N)
    exp, uniform, _, _ = dd.select_parents(fit, N, gen, seed)
    assert uniform and np.array_equal(got, exp)
    pop.close()


def test_selection_with_zero_total_fitness_is_uniform_and_flagged():
    # quadratic metric (quadratic_fitness_metric.cpp:23-28): |z| beyond s gives fitness 0 everywhere
    N, A, seed = 100, 64, 5
    pop = cg.Population(N, 1024, 1, fitness="quadratic", fit_param=1.0, mu=0.01, rho=0.0, p_neutral=0.0, seed=seed)
    rows = np.zeros((2 * N, 8), np.uint64)
    rows[:, 0] = 1  # every genome carries slot 0
    eff = np.zeros(A, np.float32)
    eff[0] = 100.0  # z = 200 per individual; s = sqrt(4 N mu) = 2
    pop.load_population(N, rows, np.linspace(0.01, 0.99, A), eff)
    fit, gen = pop.fitness(), pop.info()["generation"]
    assert np.all(fit == 0.0)
    pop.begin_generation(N, 0)
    got = pop.select(N)
    exp, uniform, _, total = dd.select_parents(fit, N, gen, seed)
    assert uniform and total == 0.0
    assert np.array_equal(got, exp)
    assert pop.info()["device_error"] & 64, "all-zero fitness must set CLOTHO_DEVERR_FITNESS"
    pop.close()


def test_parent_counts_follow_fitness_under_strong_selection(capsys):
    from scipy import stats
    rng = np.random.default_rng(2026)
    N, seed = 20_000, 31337
    pop = loaded(N, 512, 2, "gaussian_vs", 4.0, seed, rng)
    fit = pop.fitness()
    pop.begin_generation(N, 0)
    got = pop.select(N)
    pop.close()
    expected = 2.0 * N * fit / fit.sum()
    obs = np.bincount(got, minlength=N).astype(np.float64)
    # pool parents of similar fitness into bins of >= 50 expected draws
    order = np.argsort(expected)
    ce = np.cumsum(expected[order])
    edges = np.searchsorted(ce, np.arange(50.0, ce[-1], 50.0))
    e_b = np.add.reduceat(expected[order], np.r_[0, edges[:-1]])
    o_b = np.add.reduceat(obs[order], np.r_[0, edges[:-1]])
    chi2 = float(np.sum((o_b - e_b) ** 2 / e_b))
    p = float(stats.chi2.sf(chi2, len(e_b) - 1))
    top = order[-N // 10:]
    with capsys.disabled():
        print(f"\nselection chi2 = {chi2:.1f} over {len(e_b) - 1} dof, p = {p:.3f}; top decile drew "
              f"{obs[top].sum():.0f} of {2 * N} parents (expected {expected[top].sum():.0f})")
    assert p > 1e-4
    assert abs(obs[top].sum() - expected[top].sum()) < 5.0 * math.sqrt(expected[top].sum())


# ---------------------------------------------------------------------------
# whole device-drawn generations replayed through the oracle

def replay_device_generations(orc, gpu, sizes, kind, fit_param, mu, rho, bias, q1, T, p_neutral, seed,
                              compare=compare_state):
    for g, N in enumerate(sizes):
        before = gpu.info()
        fit = gpu.fitness()
        gen = before["generation"]
        gpu.simulate_philox(N)
        info = gpu.info()
        assert info["device_error"] == 0, f"gen {g}: device error {info['device_error']}"
        pairs = gpu.pairs()
        exp_pairs, _, _, _ = dd.select_parents(fit, N, gen, seed)
        assert np.array_equal(pairs, exp_pairs), f"gen {g}: parents differ from the restated draws"
        S = 2 * N
        E, swap, ev_off, ev_pos = dd.gamete_draws(S, gen, seed, rho, bias, q1, math.exp(-rho))
        mut_seq, mut_pos = dd.mutation_draws(S, gen, seed, mu, math.exp(-mu))
        M = mut_seq.size
        assert info["last_M"] == M, f"gen {g}: {info['last_M']} mutations on the device, {M} restated"
        free = gpu.free_list()
        i = np.arange(M)
        slots = np.where(i < free.size, free[np.minimum(i, max(free.size - 1, 0))] if free.size else 0,
                         before["A"] + (i - free.size))
        pos_g, _, eff_g = gpu.alleles()
        assert np.array_equal(pos_g[slots], mut_pos), f"gen {g}: new allele positions differ"
        mut_eff = eff_g[slots].astype(np.float32)
        ref = dd.mutation_effects(M, T, gen, seed, p_neutral, 0.0, 1.0)
        assert np.array_equal(mut_eff == 0.0, ref == 0.0), f"gen {g}: neutral draws differ"
        np.testing.assert_allclose(mut_eff, ref.astype(np.float32), rtol=1e-6, atol=1e-7)
        tape = oracle.Tape(N, M, pairs, swap, ev_off, ev_pos, mut_seq, mut_pos, mut_eff.reshape(-1))
        orc.step_tape(tape)
        compare(orc, gpu, g, kind=kind, fit_param=fit_param, mu=mu)


def device_pair(N_cap, A_cap, T, fitness, fit_param, mu, rho, bias, q1, p_neutral, seed, threads=4):
    orc = oracle.Oracle(T=T, fitness=FITS[fitness], fit_param=fit_param, mu=mu, rho=rho, bias=bias,
                        p_neutral=p_neutral, q1=q1, threads=threads, seed=seed)
    gpu = cg.Population(N_cap, A_cap, T, fitness=fitness, fit_param=fit_param, mu=mu, rho=rho, bias=bias,
                        p_neutral=p_neutral, q1=q1, seed=seed, max_events=int(4 * N_cap * rho + 4096),
                        max_mutations=int(4 * N_cap * mu + 4096), max_fixed=1 << 16)
    return orc, gpu


@pytest.mark.parametrize("mu", [1e-3, 0.05])
def test_bench_shape_device_generations_bit_exact(mu):
    # the N=1e6 measurement's shape at N=2,000: four traits, reference gaussian metric, rho=5,
    # 65,536-slot capacity, 58,000 pre-seeded alleles on the neutral 1/i spectrum (944-word rows)
    w = workloads.LARGE_N
    N, seed = 2000, 0xB00 + int(mu * 1e4)
    orc, gpu = device_pair(N, w.max_alleles, w.T, w.fitness, w.fit_param, mu, w.rho, 0.5, True, w.p_neutral, seed)
    pos, eff, thr = workloads.seeded_start(w, N=N)
    orc.seed_population(N, pos, eff, thr, 20261203)
    gpu.seed_population(N, pos, eff, thr, 20261203)
    assert gpu.info()["W"] == orc.info()["B"] == 912  # 58,000 slots -> 912-word rows
    replay_device_generations(orc, gpu, [N] * 4, w.fitness, w.fit_param, mu, w.rho, 0.5, True, w.T, w.p_neutral,
                              seed)


def compare_state_full_size(orc, gpu, g, kind="constant", fit_param=1.0, mu=0.0):
    """compare_state for populations whose rows take many GB on the host: rows compared in slices, and the
    phenotype bound taken from each individual's allele count n and the largest |effect| of each trait,
    (g + 2) 2^-24 max_i (n_i + 1) n_i max|w| (looser than compare_state's, which unpacks every set bit to sum
    the |w| of each individual).  Returns the largest phenotype error and the bound."""
    oi, gi = orc.info(), gpu.info()
    assert gi["device_error"] == 0, f"gen {g}: device error {gi['device_error']}"
    for k in ("N", "A", "fixed_count", "lost_count", "free_count", "fixed_total", "generation"):
        assert oi[k] == gi[k], f"gen {g}: {k} oracle={oi[k]} gpu={gi[k]}"
    assert oi["B"] == gi["W"], f"gen {g}: width oracle={oi['B']} gpu={gi['W']}"
    rg = gpu.rows()
    ro = orc.rows()
    assert ro.shape == rg.shape
    step = 1 << 16
    for r0 in range(0, rg.shape[0], step):
        a, b = ro[r0:r0 + step], rg[r0:r0 + step]
        if not np.array_equal(a, b):
            r, w = np.argwhere(a != b)[0]
            raise AssertionError(f"gen {g}: rows differ; first row {r0 + r} word {w}: "
                                 f"oracle {int(a[r, w]):#x} gpu {int(b[r, w]):#x}")
    del ro, rg
    assert np.array_equal(orc.free_list(), gpu.free_list()), f"gen {g}: free list differs"
    po, ao, eo = orc.alleles()
    pg, ag, eg = gpu.alleles()
    assert np.array_equal(po, pg) and np.array_equal(ao, ag), f"gen {g}: allele table differs"
    assert np.array_equal(eo, eg.astype(np.float64)), f"gen {g}: trait table differs"
    fpo, fao, feo = orc.fixed()
    fpg, fag, feg = gpu.fixed()
    assert np.array_equal(fpo, fpg) and np.array_equal(fao, fag) and np.array_equal(feo, feg.astype(np.float64))
    zo, zg = orc.phenotypes(), gpu.phenotypes().astype(np.float64)
    _, rowc = gpu.margins()
    n = rowc[0::2].astype(np.float64) + rowc[1::2]
    maxw = np.abs(eg.astype(np.float64)).max(axis=0)
    bound = (g + 2.0) * 2.0 ** -24 * ((n + 1.0) * n).max() * maxw + 1e-30
    err = np.abs(zo - zg)
    assert np.all(err <= bound), f"gen {g}: phenotype error {err.max()} above {bound}"
    np.testing.assert_allclose(gpu.fitness(), fitness_of(gpu.phenotypes(), kind, fit_param, gi["N"], mu),
                               rtol=1e-12, atol=1e-300)
    return float(err.max()), float(bound.max())


@pytest.mark.parametrize("mode", ["device", "tape"])
def test_bench_configuration_at_full_size_bit_exact(mode, capsys):
    # the N=1e6 measurement itself: 2e6 rows of 912 words, 58,000 pre-seeded alleles, four traits, the
    # reference gaussian metric, rho=5, mu=1e-3, with the measurement's seed and capacities, two generations
    # against the oracle on every host core: device-drawn parents, breakpoints and mutations replayed through
    # the oracle ("device"), or the drop-in's event tape drawn by the oracle's recorder ("tape")
    import os
    w = workloads.LARGE_N
    N, seed = w.N, 20261203
    gpu = cg.Population(N, w.max_alleles, w.T, fitness=w.fitness, fit_param=w.fit_param, mu=w.mu, rho=w.rho,
                        bias=w.bias, p_neutral=w.p_neutral, seed=seed, max_fixed=1 << 20,
                        max_events=int(2 * N * w.rho * 1.05 + 4096), max_mutations=int(2 * N * w.mu * 1.5 + 4096))
    orc = oracle.Oracle(T=w.T, fitness=FITS[w.fitness], fit_param=w.fit_param, mu=w.mu, rho=w.rho, bias=w.bias,
                        p_neutral=w.p_neutral, q1=True, threads=os.cpu_count() or 4, seed=seed)
    pos, eff, thr = workloads.seeded_start(w)
    gpu.seed_population(N, pos, eff, thr, seed)
    rows = gpu.rows()
    assert rows.shape == (2 * N, 912)
    orc.load_population(N, rows, pos, eff)
    del rows
    errs = []

    def compare(orc_, gpu_, g, **kw):
        errs.append(compare_state_full_size(orc_, gpu_, g, **kw))

    if mode == "device":
        replay_device_generations(orc, gpu, [N] * 2, w.fitness, w.fit_param, w.mu, w.rho, w.bias, True, w.T,
                                  w.p_neutral, seed, compare=compare)
    else:
        for g in range(2):
            gpu.simulate(orc.step_record(N))
            compare(orc, gpu, g, kind=w.fitness, fit_param=w.fit_param, mu=w.mu)
    with capsys.disabled():
        print(f"\nN=1e6 measurement workload, 2 {mode} generations: rows bit-exact; phenotype "
              f"|FP32 carried - FP64| max {max(e for e, _ in errs):.3e} (bound {min(b for _, b in errs):.3e}), "
              f"alleles {gpu.info()['A']}, row width {gpu.info()['W']} words")
    orc.close()
    gpu.close()


@pytest.mark.parametrize("case", ["qtl_selection", "q1_off_quadratic", "chunk_masks", "many_breakpoints",
                                  "interval_classifier", "size_changes"])
def test_device_generations_bit_exact(case):
    if case == "qtl_selection":      # C2-shaped: one trait, N(0,1) effects, exp(-z^2/2)
        kw = dict(T=1, fitness="gaussian_vs", fit_param=1.0, mu=0.1, rho=1.0, bias=0.5, q1=True, p_neutral=0.0)
        sizes, A_cap = [500] * 25, 8192
    elif case == "q1_off_quadratic":
        kw = dict(T=3, fitness="quadratic", fit_param=3.0, mu=0.2, rho=3.0, bias=0.3, q1=False, p_neutral=0.5)
        sizes, A_cap = [200] * 15, 8192
    elif case == "chunk_masks":           # capacity above 65,536 slots, rho <= 1: masks chunk by chunk
        kw = dict(T=2, fitness="gaussian_vs", fit_param=4.0, mu=0.5, rho=1.0, bias=0.5, q1=False, p_neutral=0.5)
        sizes, A_cap = [100] * 8, 70_000
    elif case == "many_breakpoints":      # rho = 20 (interval classifier): most rows have > 16 breakpoints
        kw = dict(T=1, fitness="gaussian_vs", fit_param=4.0, mu=0.5, rho=20.0, bias=0.5, q1=False, p_neutral=0.5)
        sizes, A_cap = [80] * 6, 70_000
    elif case == "interval_classifier":   # capacity above 524,288 slots
        kw = dict(T=2, fitness="gaussian_vs", fit_param=4.0, mu=0.5, rho=3.0, bias=0.5, q1=True, p_neutral=0.5)
        sizes, A_cap = [100] * 8, 600_000
    else:                                 # growth, a fall below half, a one-individual bottleneck, regrowth
        kw = dict(T=2, fitness="gaussian", fit_param=1.0, mu=0.3, rho=2.0, bias=0.5, q1=False, p_neutral=0.2)
        sizes, A_cap = [300, 450, 120, 1, 50, 400, 400], 8192
    seed = 0xD0 + len(case)
    orc, gpu = device_pair(max(sizes), A_cap, seed=seed, **kw)
    orc.init(sizes[0])
    gpu.init(sizes[0])
    replay_device_generations(orc, gpu, sizes, kw["fitness"], kw["fit_param"], kw["mu"], kw["rho"], kw["bias"],
                              kw["q1"], kw["T"], kw["p_neutral"], seed)
    assert gpu.info()["A"] > 0


# ---------------------------------------------------------------------------
# statistics of device-drawn runs against oracle runs with the oracle's own draws

LOG2_BINS = 8


def spectrum_stats(rows, A, fit):
    """(binned SFS by log2 carrier count, segregating sites, heterozygosity, mean fitness)
    from the rows: column margins as population_space_row_frequency_evaluator.hpp:37-62."""
    S = rows.shape[0]
    bits = np.unpackbits(rows.view(np.uint8).reshape(S, -1), axis=1, bitorder="little")[:, :A]
    c = bits.sum(axis=0)
    seg = (c > 0) & (c < S)
    b = np.floor(np.log2(np.maximum(c[seg], 1))).astype(int)
    sfs = np.bincount(np.minimum(b, LOG2_BINS - 1), minlength=LOG2_BINS)
    f = c / S
    return sfs, int(seg.sum()), float(np.sum(2.0 * f * (1.0 - f))), float(np.mean(fit))


def test_device_runs_match_oracle_runs_in_distribution(capsys):
    # the bench workload's shape (four traits, reference gaussian metric, rho=5, pre-seeded 1/i load)
    # at N=1,000 with mu=0.01 so that 20 new alleles arrive each generation
    # Bound: each statistic's replicate means within 5 standard errors (the naive ones, from the replicate
    # variances).  Those understate the spread of the carrier-count bins: on the CPU, with the device's draw
    # rules replayed through the oracle, arms drawing from one law (two seed families of either generator,
    # 256 replicates each) differed by up to 3.0 of them on the 4-7 carrier bin, while the two laws pooled
    # agreed there (26.80 against 27.08 sites, z = -0.9).  Exact agreement is what the replays above
    # establish; this guards the laws themselves.
    w = workloads.LARGE_N
    N, mu, G, R = 1000, 0.01, 60, 96
    S = 2 * N
    rng = np.random.default_rng(99)
    A0 = 330  # ~ theta * H(S-1) with theta = 4 N mu = 40
    pos = rng.random(A0)
    eff = rng.standard_normal(A0 * w.T).astype(np.float32)
    thr = workloads.neutral_spectrum_thresholds(rng, S, A0)
    dev, orc = [], []
    for r in range(R):
        gpu = cg.Population(N, 8192, w.T, fitness=w.fitness, fit_param=w.fit_param, mu=mu, rho=w.rho,
                            p_neutral=w.p_neutral, seed=20000 + 7 * r, max_events=int(4 * N * w.rho + 4096),
                            max_mutations=4096, max_fixed=1 << 14)
        gpu.seed_population(N, pos, eff, thr, 7)
        gpu.run_philox(N, G)
        gpu.check()
        rows, A = gpu.rows(), gpu.info()["A"]
        st = gpu.stats(sfs_len=S + 1)
        # the library's own statistics equal the ones computed here from its rows
        col = np.unpackbits(rows.view(np.uint8).reshape(S, -1), axis=1, bitorder="little")[:, :A].sum(axis=0)
        assert st["segregating"] == int(np.sum((col > 0) & (col < S)))
        assert np.array_equal(st["sfs"][:S + 1], np.bincount(col, minlength=S + 1)[:S + 1])
        f = col / S
        assert abs(st["heterozygosity"] - np.sum(2 * f * (1 - f))) <= 1e-9 * max(1.0, st["heterozygosity"])
        fit = gpu.fitness()
        assert abs(st["mean_fitness"] - fit.mean()) <= 1e-12 * fit.mean()
        dev.append(spectrum_stats(rows, A, fit))
        gpu.close()
        o = oracle.Oracle(T=w.T, fitness=FITS[w.fitness], fit_param=w.fit_param, mu=mu, rho=w.rho,
                          p_neutral=w.p_neutral, threads=1, seed=90000 + 13 * r)
        o.seed_population(N, pos, eff, thr, 7)
        for _ in range(G):
            o.step_record(N)
        orc.append(spectrum_stats(o.rows(), o.info()["A"], o.fitness()))
        o.close()
    lines = []
    for name, k in (("segregating", 1), ("heterozygosity", 2), ("mean_fitness", 3)):
        a = np.array([d[k] for d in dev], np.float64)
        b = np.array([d[k] for d in orc], np.float64)
        se = math.sqrt(a.var(ddof=1) / R + b.var(ddof=1) / R)
        lines.append(f"{name}: device {a.mean():.4g} oracle {b.mean():.4g} (se {se:.3g})")
        assert abs(a.mean() - b.mean()) <= 5.0 * se + 1e-12 * abs(b.mean()), lines[-1]
    sa = np.array([d[0] for d in dev], np.float64)
    sb = np.array([d[0] for d in orc], np.float64)
    for j in range(5):  # carrier counts 1, 2-3, 4-7, 8-15, 16-31
        se = math.sqrt(sa[:, j].var(ddof=1) / R + sb[:, j].var(ddof=1) / R)
        lines.append(f"sfs bin {j}: device {sa[:, j].mean():.2f} oracle {sb[:, j].mean():.2f} (se {se:.2f})")
        assert abs(sa[:, j].mean() - sb[:, j].mean()) <= 5.0 * se, lines[-1]
    with capsys.disabled():
        print("\ndevice-drawn vs oracle runs (N=1,000, G=60, 96 replicates each):\n  " + "\n  ".join(lines))
