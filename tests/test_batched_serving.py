"""Batched and served forms: many populations per launch, continuous batching.
Every population's draws depend only on its own seed and generation, so its
genomes and statistics must be bit-identical alone and in the mix."""
import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu

if not gpu_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import clotho_gb300 as cg  # noqa: E402
from clotho_gb300 import serving, autotune  # noqa: E402

SPECS = [
    dict(N=700, T=1, mu=0.05, rho=0.5, fitness="constant", seed=11),
    dict(N=3000, T=4, mu=0.01, rho=5.0, fitness="gaussian", seed=12),
    dict(N=150, T=2, mu=0.2, rho=1.0, fitness="gaussian_vs", fit_param=20.0, seed=13),
    dict(N=1200, T=3, mu=0.02, rho=2.0, fitness="quadratic", fit_param=5.0, seed=14),
    dict(N=64, T=1, mu=0.5, rho=0.1, fitness="gaussian_vs", fit_param=2.0, seed=15),
]


def desc_of(s):
    kw = {k: v for k, v in s.items() if k not in ("N", "T")}
    return cg.make_desc(s["N"], 1 << 14, s["T"], p_neutral=0.3, **kw)


def alone(s, G):
    d = desc_of(s)
    pop = cg.Population(s["N"], 1 << 14, s["T"], mu=s["mu"], rho=s["rho"], fitness=s["fitness"],
                        fit_param=s.get("fit_param", 1.0), p_neutral=0.3, seed=s["seed"], max_events=d.max_events,
                        max_mutations=d.max_mutations, max_fixed=d.max_fixed)
    pop.init(s["N"])
    pop.run_philox(s["N"], G)
    pop.check()
    return pop.rows(), pop.stats(64)


def test_batch_equals_alone():
    G = 25
    b = cg.Batch([desc_of(s) for s in SPECS])
    b.init()
    b.run(G)
    b.sync()
    for i, s in enumerate(SPECS):
        assert b.info(i)["device_error"] == 0
        rows, st = alone(s, G)
        assert np.array_equal(b.rows(i), rows), i
        bs = b.stats(i, 64)
        assert bs["segregating"] == st["segregating"] and np.array_equal(bs["sfs"], st["sfs"])
        assert bs["mean_fitness"] == st["mean_fitness"]


def test_narrow_and_wide_builds_agree():
    # 512 slots (8-word rows): alone the population runs the narrow build of the generation kernel; batched
    # with a population of 256-word rows it runs the wide build.  Same rows, spectrum and mean fitness.
    G = 20
    s = dict(N=500, T=2, mu=0.01, rho=3.0, fitness="gaussian_vs", fit_param=20.0, seed=21)
    kw = {k: v for k, v in s.items() if k not in ("N", "T")}
    d = cg.make_desc(s["N"], 512, s["T"], p_neutral=0.3, **kw)
    pop = cg.Population(s["N"], 512, s["T"], mu=s["mu"], rho=s["rho"], fitness=s["fitness"],
                        fit_param=s["fit_param"], p_neutral=0.3, seed=s["seed"], max_events=d.max_events,
                        max_mutations=d.max_mutations, max_fixed=d.max_fixed)
    pop.init(s["N"])
    pop.run_philox(s["N"], G)
    pop.check()
    b = cg.Batch([d, desc_of(SPECS[1])])
    b.init()
    b.run(G)
    assert b.info(0)["device_error"] == 0
    assert np.array_equal(b.rows(0), pop.rows())
    bs, st = b.stats(0, 64), pop.stats(64)
    assert np.array_equal(bs["sfs"], st["sfs"]) and bs["mean_fitness"] == st["mean_fitness"]
    # row capacities (512 and 16,384 slots: 8 and 256 words) decide the build, not the live widths
    assert d.max_alleles <= 128 * 64 < desc_of(SPECS[1]).max_alleles


def test_each_population_keeps_its_classifier_in_a_mixed_batch():
    # a batch holding a population of more than 524,288 slots (interval classifier) and a small one (suffix
    # table): the generation kernel runs one pass per classifier, so each population runs the classifier it
    # runs alone and its rows, spectrum and fitness are bit-identical to its run alone
    G = 15
    small = dict(N=400, T=2, mu=0.02, rho=4.0, fitness="gaussian_vs", fit_param=20.0, seed=31)
    big = dict(N=300, T=1, mu=0.05, rho=2.0, fitness="constant", fit_param=1.0, seed=32)
    caps = (4096, 600_000)
    descs, alone = [], []
    for s, cap in zip((small, big), caps):
        kw = {k: v for k, v in s.items() if k not in ("N", "T")}
        d = cg.make_desc(s["N"], cap, s["T"], p_neutral=0.3, **kw)
        descs.append(d)
        pop = cg.Population(s["N"], cap, s["T"], mu=s["mu"], rho=s["rho"], fitness=s["fitness"],
                            fit_param=s["fit_param"], p_neutral=0.3, seed=s["seed"], max_events=d.max_events,
                            max_mutations=d.max_mutations, max_fixed=d.max_fixed)
        pop.init(s["N"])
        pop.run_philox(s["N"], G)
        pop.check()
        alone.append(pop)
    b = cg.Batch(descs)
    b.init()
    b.run(G)
    for i, pop in enumerate(alone):
        assert b.info(i)["device_error"] == 0
        assert np.array_equal(b.rows(i), pop.rows())
        bs, st = b.stats(i, 64), pop.stats(64)
        assert np.array_equal(bs["sfs"], st["sfs"])
        assert bs["mean_fitness"] == st["mean_fitness"]
        assert b.info(i)["mean_fitness"] == pop.info()["mean_fitness"]
    b.close()


def test_shared_and_global_accumulators_in_one_batch():
    # an interval-classifier population (1.2e6 slots) whose rows pass 6,976 words in its first generation
    # (480,000 new alleles: 40 individuals, mu = 6,000 per sequence) folds into its global AND/OR
    # accumulators, batched with a 73,728-slot population (chunk-mask build) and a 4,096-slot one (bitmap
    # build): three passes of the generation kernel over the same items, and each population's rows,
    # spectrum and fitness equal its run alone
    G = 3
    specs = [(dict(N=40, T=1, mu=6000.0, rho=2.0, fitness="gaussian_vs", fit_param=50.0, seed=41), 1_200_000),
             (dict(N=300, T=1, mu=0.05, rho=1.0, fitness="constant", fit_param=1.0, seed=42), 70_000),
             (dict(N=400, T=2, mu=0.02, rho=4.0, fitness="gaussian_vs", fit_param=20.0, seed=43), 4096)]
    descs, alone = [], []
    for s, cap in specs:
        kw = {k: v for k, v in s.items() if k not in ("N", "T")}
        d = cg.make_desc(s["N"], cap, s["T"], p_neutral=0.3, **kw)
        descs.append(d)
        pop = cg.Population(s["N"], cap, s["T"], mu=s["mu"], rho=s["rho"], fitness=s["fitness"],
                            fit_param=s["fit_param"], p_neutral=0.3, seed=s["seed"], max_events=d.max_events,
                            max_mutations=d.max_mutations, max_fixed=d.max_fixed)
        pop.init(s["N"])
        pop.run_philox(s["N"], G)
        pop.check()
        alone.append(pop)
    assert alone[0].info()["W"] > 6976
    b = cg.Batch(descs)
    b.init()
    b.run(G)
    for i, pop in enumerate(alone):
        assert b.info(i)["device_error"] == 0
        assert np.array_equal(b.rows(i), pop.rows()), i
        bs, st = b.stats(i, 64), pop.stats(64)
        assert np.array_equal(bs["sfs"], st["sfs"])
        assert bs["mean_fitness"] == st["mean_fitness"]
    b.close()


@pytest.mark.parametrize("cap", [8192, 1 << 14, 70_000])
def test_launch_shapes_do_not_change_results(cap):
    # every tuning knob (rows per item, the narrow build where rows are at most 128 words, blocks per SM of
    # the per-individual kernels) gives bit-identical rows, statistics and mean fitness; at 8,192 slots
    # the narrow build runs unless switched off; at 70,000 slots the populations of rho <= 1 run the
    # chunk-mask build and the other one the interval classifier
    G = 6
    outs = []
    for rpi, narrow, blocks in ((64, 1, 16), (1024, 0, 4), (256, 1, 24), (512, 0, 8)):
        b = cg.Batch([cg.make_desc(s["N"], cap, s["T"], p_neutral=0.3,
                                   **{k: v for k, v in s.items() if k not in ("N", "T")}) for s in SPECS[:3]])
        b.init()
        b.set_tuning(rows_per_item=rpi, narrow_build=narrow, row_blocks_per_sm=blocks)
        assert b.tuning() == {"rows_per_item": rpi, "narrow_build": narrow, "row_blocks_per_sm": blocks}
        b.run(G)
        outs.append([(b.rows(i), b.stats(i, 64), b.info(i)) for i in range(3)])
        b.close()
    for other in outs[1:]:
        for (ra, sa, ia), (rb, sb, ib) in zip(outs[0], other):
            assert ia["device_error"] == 0 and ib["device_error"] == 0
            assert np.array_equal(ra, rb)
            assert np.array_equal(sa["sfs"], sb["sfs"]) and sa["mean_fitness"] == sb["mean_fitness"]


def test_autotuner_picks_a_candidate(tmp_path):
    b = cg.Batch([desc_of(s) for s in SPECS])
    b.init()
    best = autotune.tune(b, gens_per_trial=1, cache_path=str(tmp_path / "tune.json"))
    assert set(best) == set(autotune.DEFAULT)
    assert all(best[k] in v for k, v in autotune.CANDIDATES.items())
    assert b.tuning() == best
    assert autotune.tune(b, cache_path=str(tmp_path / "tune.json")) == best  # cached


def test_serving_results_match_plain_engine():
    jobs = serving.synthetic_jobs(10, rate=200.0, seed=3, N_range=(200, 3000), G_range=(10, 40))
    plain = [serving.Job(**{k: getattr(j, k) for k in ("id", "N", "mu", "rho", "T", "G", "seed", "arrival")})
             for j in jobs]
    srv = serving.Server(budget_bytes=8 << 30, max_slots=4)
    s1 = srv.run_open_loop(jobs)
    s2 = serving.run_plain(plain)
    assert s1["jobs"] == s2["jobs"] == 10 and s1["errors"] == 0
    by_id = {j.id: j for j in plain}
    for j in srv.finished:
        a, b = j.result, by_id[j.id].result
        assert a["sfs"] == b["sfs"] and a["segregating"] == b["segregating"]
        assert a["mean_fitness"] == b["mean_fitness"] and a["generation"] == b["generation"] == j.G


def test_admission_waits_for_memory():
    jobs = serving.synthetic_jobs(4, rate=1000.0, seed=5, N_range=(500, 600), G_range=(5, 5))
    one = cg.footprint_of(jobs[0].desc())
    srv = serving.Server(budget_bytes=int(one * 1.5), max_slots=8)   # room for one job at a time
    s = srv.run_open_loop(jobs)
    assert s["jobs"] == 4 and s["errors"] == 0
    # never more than one resident: admissions are strictly after the previous job finished
    fin = sorted(srv.finished, key=lambda j: j.admitted)
    for a, b in zip(fin, fin[1:]):
        assert b.admitted >= a.done - 1e-6


def wf_sojourn(n):
    """Expected generations an allele born in one of n sequences spends at each count 1..n-1 (count at
    birth included) under neutral Wright-Fisher resampling, counts i -> Binomial(n, i/n): row 1 of
    (I - Q)^-1 over the transient counts."""
    from math import lgamma, log, exp
    i = np.arange(1, n)
    lc = np.array([lgamma(n + 1) - lgamma(j + 1) - lgamma(n - j + 1) for j in range(1, n)])
    Q = np.empty((n - 1, n - 1))
    for a in range(1, n):
        p = a / n
        Q[a - 1] = np.exp(lc + i * log(p) + (n - i) * log(1.0 - p))
    e1 = np.zeros(n - 1)
    e1[0] = 1.0
    return np.linalg.solve((np.eye(n - 1) - Q).T, e1)


def test_device_draws_match_neutral_theory():
    # Device-drawn (Philox) generations have no bit parity with the reference's Boost stream, so they are
    # checked against the neutral Wright-Fisher expectation with infinite sites: 2N mu new alleles a
    # generation, each resampled Binomial(2N, i/2N) (every sequence copies a random parent strand at a
    # neutral site); sites carried by i sequences = 2N mu x the expected generations at count i.  (The
    # diffusion limit theta / i, theta = 4 N mu, undercounts singletons by about 13% at 2N = 400.)
    # 64 replicates in one batch, 8N generations of burn-in from an empty start, then 20 samples N/4
    # generations apart.
    N, mu, rho, R = 200, 0.05, 0.5, 64
    b = cg.Batch([cg.make_desc(N, 8192, 1, mu=mu, rho=rho, p_neutral=1.0, fitness="constant", seed=1000 + r)
                  for r in range(R)])
    b.init()
    b.run(8 * N)
    seg, sfs = [], []
    for _ in range(20):
        b.run(N // 4)
        for i in range(R):
            st = b.stats(i, 2 * N + 1)
            assert b.info(i)["device_error"] == 0
            seg.append(st["segregating"])
            sfs.append(st["sfs"][1:4].astype(np.float64))
    xi_expect = 2 * N * mu * wf_sojourn(2 * N)
    assert abs(np.mean(seg) / xi_expect.sum() - 1.0) < 0.06, (np.mean(seg), xi_expect.sum())
    xi = np.mean(sfs, axis=0)                      # sites carried by 1, 2, 3 sequences
    assert np.all(np.abs(xi / xi_expect[:3] - 1.0) < 0.05), (xi, xi_expect[:3])
    b.close()


def _columns(rows, A):
    S = rows.shape[0]
    return np.unpackbits(rows.view(np.uint8).reshape(S, -1), axis=1, bitorder="little")[:, :A].sum(axis=0)


@pytest.mark.parametrize("cap", [8192, 1 << 14])
def test_fused_column_counts_equal_the_rows(cap):
    # populations that count their columns inside the generation step (bit-sliced counters in the kernel's
    # shared memory): their statistics, read from those counts, equal numpy over their rows and the
    # on-demand pass over the rows; counting changes no row, and the populations that do not count are
    # untouched (8,192 slots: the narrow build; 16,384: the wide one)
    G = 5
    descs = [cg.make_desc(s["N"], cap, s["T"], p_neutral=0.3, **{k: v for k, v in s.items() if k not in ("N", "T")})
             for s in SPECS]
    a = cg.Batch(descs)
    a.init()
    b = cg.Batch(descs)
    b.init()
    for i in (0, 1, 3):
        a.count_columns(i)
    a.run(G)
    b.run(G)
    for i in range(len(SPECS)):
        ra = a.rows(i)
        assert np.array_equal(ra, b.rows(i)) and a.info(i)["device_error"] == 0
        S, A = ra.shape[0], a.info(i)["A"]
        col = _columns(ra, A)
        sa, sb = a.stats(i, S + 1), b.stats(i, S + 1)
        assert np.array_equal(sa["sfs"], np.bincount(col, minlength=S + 1)[:S + 1])
        assert np.array_equal(sa["sfs"], sb["sfs"])
        assert sa["segregating"] == int(((col > 0) & (col < S)).sum())
        f = col / S
        assert abs(sa["heterozygosity"] - np.sum(2 * f * (1 - f))) <= 1e-9 * max(1.0, sa["heterozygosity"])
        assert sa["mean_fitness"] == sb["mean_fitness"]
        mcol, _ = a.margins(i)   # the on-demand pass
        assert np.array_equal(mcol, col)
    a.close()
    b.close()


def test_fused_column_counts_of_one_population():
    s = SPECS[1]
    d = desc_of(s)
    pop = cg.Population(s["N"], 1 << 14, s["T"], mu=s["mu"], rho=s["rho"], fitness=s["fitness"], p_neutral=0.3,
                        seed=s["seed"], max_events=d.max_events, max_mutations=d.max_mutations)
    pop.init(s["N"])
    pop.count_columns()
    pop.run_philox(s["N"], 6)
    pop.check()
    rows = pop.rows()
    S, A = rows.shape[0], pop.info()["A"]
    col = _columns(rows, A)
    st = pop.stats(S + 1)
    assert np.array_equal(st["sfs"], np.bincount(col, minlength=S + 1)[:S + 1])
    assert abs(st["mean_fitness"] - pop.fitness().mean()) <= 1e-12 * pop.fitness().mean()
    pop.count_columns(False)
    pop.run_philox(s["N"], 1)
    rows = pop.rows()
    assert np.array_equal(pop.stats(S + 1)["sfs"], np.bincount(_columns(rows, pop.info()["A"]), minlength=S + 1)[:S + 1])


def test_served_job_results_match_numpy_on_the_rows():
    # every field of a served job's result -- the 64-bin spectrum (counted inside its last chunk of
    # generations), segregating sites, mean fitness, generation, device error -- against numpy over the same
    # job run alone
    jobs = serving.synthetic_jobs(12, rate=500.0, seed=8, N_range=(200, 3000), G_range=(5, 30))
    srv = serving.Server(budget_bytes=8 << 30, max_slots=5)
    srv.run_open_loop(jobs)
    assert len(srv.finished) == 12
    for j in srv.finished:
        d = j.desc()
        pop = cg.Population(j.N, j.max_alleles(), j.T, mu=j.mu, rho=j.rho, fitness=j.fitness, fit_param=j.fit_param,
                            p_neutral=j.p_neutral, seed=j.seed, max_events=d.max_events,
                            max_mutations=d.max_mutations, max_fixed=d.max_fixed)
        pop.init(j.N)
        pop.run_philox(j.N, j.G)
        rows = pop.rows()
        S, A = rows.shape[0], pop.info()["A"]
        col = _columns(rows, A)
        sfs = np.bincount(np.minimum(col, 63), minlength=64)[:64]
        fit = pop.fitness()
        r = j.result
        assert r["sfs"] == sfs.tolist(), j.id
        assert r["segregating"] == int(((col > 0) & (col < S)).sum())
        assert abs(r["mean_fitness"] - fit.mean()) <= 1e-12 * max(1.0, abs(fit.mean()))
        assert r["generation"] == j.G and r["device_error"] == 0
        pop.close()
