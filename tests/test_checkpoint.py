"""Checkpoint / resume and population margins through the C-ABI.

A population saved between generations and restored into a fresh context
continues exactly as the uninterrupted run: device-drawn generations are keyed
by (seed, generation), so rows, phenotypes and fitness are bit-identical, and a
tape-driven run stays bit-exact against the oracle after the restore.
"""
import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = pytest.mark.gpu

if not gpu_available():  # collected on CPU machines, skipped there
    pytest.skip("no CUDA device", allow_module_level=True)

import clotho_gb300 as cg  # noqa: E402
from tests.test_gpu_parity import compare_state, make_pair  # noqa: E402

KW = dict(fitness="gaussian_vs", fit_param=3.0, mu=0.05, rho=2.0, p_neutral=0.3, seed=77,
          max_events=1 << 15, max_mutations=1 << 13, max_fixed=1 << 14)


def _state(pop):
    i = pop.info()
    return pop.rows(), pop.phenotypes(), pop.fitness(), pop.alleles(), pop.fixed(), i


def _same(a, b):
    ra, pa, fa, (posa, agea, effa), (fpa, faa, fea), ia = a
    rb, pb, fb, (posb, ageb, effb), (fpb, fab, feb), ib = b
    assert ia == ib
    assert np.array_equal(ra, rb)
    assert np.array_equal(pa, pb) and np.array_equal(fa, fb)
    assert np.array_equal(posa, posb) and np.array_equal(agea, ageb) and np.array_equal(effa, effb)
    assert np.array_equal(fpa, fpb) and np.array_equal(faa, fab) and np.array_equal(fea, feb)


def test_resume_device_drawn_run_is_bit_identical(tmp_path):
    N = 1500
    a = cg.Population(N, 1 << 13, 2, **KW)
    a.init(N)
    for _ in range(6):
        a.simulate_philox(N)
    snap = a.snapshot()
    a.save(str(tmp_path / "pop.ckpt"))
    a.run_philox(N, 5)
    a.check()
    ref = _state(a)

    b = cg.Population(N, 1 << 13, 2, **KW)  # fresh context, same parameters
    b.restore(snap)
    assert b.info()["generation"] == 7
    b.run_philox(N, 5)
    b.check()
    _same(ref, _state(b))

    c = cg.Population(2 * N, 1 << 14, 2, **KW)  # larger capacities hold it too; restored from the file
    c.load(str(tmp_path / "pop.ckpt"))
    for _ in range(5):
        c.simulate_philox(N)
    _same(ref, _state(c))
    for p in (a, b, c):
        p.close()


def test_resume_tape_run_stays_bit_exact_against_the_oracle():
    N = 200
    orc, gpu = make_pair(N, 8192, T=2, fitness="gaussian_vs", fit_param=4.0, mu=0.2, rho=1.5, p_neutral=0.4)
    orc.init(N)
    gpu.init(N)
    for g in range(6):
        gpu.simulate(orc.step_record(N))
    snap = gpu.snapshot()
    gpu.close()
    _, fresh = make_pair(N, 8192, T=2, fitness="gaussian_vs", fit_param=4.0, mu=0.2, rho=1.5, p_neutral=0.4)
    fresh.restore(snap)
    compare_state(orc, fresh, 5, kind="gaussian_vs", fit_param=4.0)
    for g in range(6, 12):
        fresh.simulate(orc.step_record(N))
        compare_state(orc, fresh, g, kind="gaussian_vs", fit_param=4.0)
    fresh.close()


def test_restore_rejects_other_parameters_and_damaged_snapshots():
    N = 300
    a = cg.Population(N, 4096, 2, **KW)
    a.init(N)
    a.run_philox(N, 3)
    snap = a.snapshot()
    other = cg.Population(N, 4096, 2, **dict(KW, rho=2.5))
    with pytest.raises(cg.ClothoError):
        other.restore(snap)
    small = cg.Population(N // 2, 4096, 2, **KW)
    with pytest.raises(cg.ClothoError):
        small.restore(snap)
    same = cg.Population(N, 4096, 2, **KW)
    with pytest.raises(cg.ClothoError):
        same.restore(snap[: len(snap) // 2])
    with pytest.raises(cg.ClothoError):
        same.restore(b"\0" * len(snap))
    same.restore(snap)  # the intact snapshot still works after the refusals
    assert same.info()["generation"] == a.info()["generation"]
    for p in (a, other, small, same):
        p.close()


def test_margins_and_allele_frequency_log_match_the_rows():
    N = 800
    pop = cg.Population(N, 1 << 13, 1, **dict(KW, mu=0.3))
    pop.init(N)
    pop.run_philox(N, 15)
    i = pop.info()
    rows = pop.rows()
    bits = np.unpackbits(rows.view(np.uint8).reshape(rows.shape[0], -1), axis=1, bitorder="little")
    col, row = pop.margins()
    assert np.array_equal(col, bits[:, : i["A"]].sum(axis=0))
    assert np.array_equal(row, bits.sum(axis=1))
    log = pop.allele_frequency_log()
    assert log["distribution"] == [int(x) for x in col]
    freq = log["frequency_distribution"]
    assert len(freq) == 2 * N + 1 and sum(freq) == i["A"]
    st = pop.stats(sfs_len=2 * N + 1)
    assert np.array_equal(np.asarray(freq), st["sfs"])
    assert st["segregating"] == int(((col > 0) & (col < 2 * N)).sum())
    assert log["stats"]["alleles_per_sequence"]["total"] == 2 * N
    assert log["stats"]["sequences_per_allele"]["max"] == int(col.max())
    pop.close()


def test_pairwise_difference_matches_numpy():
    N = 700
    pop = cg.Population(N, 1 << 13, 1, **dict(KW, mu=0.3))
    pop.init(N)
    pop.run_philox(N, 12)
    rows = pop.rows()
    bits = np.unpackbits(rows.view(np.uint8).reshape(rows.shape[0], -1), axis=1, bitorder="little").astype(np.int32)
    rng = np.random.default_rng(9)
    for sample in (rng.choice(2 * N, 150, replace=False), np.arange(65), np.arange(2 * N)):
        sub = bits[sample]
        d = (sub[:, None, :] != sub[None, :, :]).sum(axis=2) if len(sample) <= 200 else None
        got = pop.pairwise_difference(sample=sample, distances=len(sample) <= 200)
        n = len(sample)
        assert got["count"] == n * (n - 1) // 2
        if d is not None:
            iu = np.triu_indices(n, 1)
            ref = d[iu]
            assert np.array_equal(got["distances"], ref)     # row-major upper triangle
            assert got["total"] == ref.sum() and got["min"] == ref.min() and got["max"] == ref.max()
            assert abs(got["mean"] - ref.mean()) < 1e-9 and abs(got["variance"] - ref.var()) < 1e-6
            assert got["median"] == float(np.median(ref))
        else:
            # totals from per-site counts: sum over pairs = sum over sites of c (n - c)
            c = sub.sum(axis=0).astype(np.int64)
            assert got["total"] == int((c * (n - c)).sum())
    pop.close()


def test_growth_schedule_in_one_graph_equals_generation_by_generation():
    from clotho_gb300 import growth
    sizes = growth.schedule(growth.LinearGrowth(1.2, 7.0), 300, 1, 8)
    kw = dict(KW, max_events=1 << 16, max_mutations=1 << 13)
    a = cg.Population(2000, 1 << 13, 2, **kw)
    b = cg.Population(2000, 1 << 13, 2, **kw)
    for p in (a, b):
        p.init(300)
    a.run_philox_schedule(sizes)
    for n in sizes:
        b.simulate_philox(n)
    a.check()
    assert a.info()["N"] == sizes[-1]
    _same(_state(a), _state(b))
    # a predefined schedule on a batch of two populations
    bt = cg.Batch([a.desc, a.desc])
    bt.N = [200, 200]
    bt.init()
    sched = [[100 + 10 * g, 400 - 20 * g] for g in range(6)]
    bt.run_schedule(sched)
    assert [bt.info(i)["N"] for i in range(2)] == sched[-1]
    assert all(bt.info(i)["device_error"] == 0 for i in range(2))
    for p in (a, b):
        p.close()
    bt.close()


def test_batch_schedules_that_shrink_match_populations_run_alone():
    # per-population sizes that shrink more than tenfold in one generation and regrow, on a batch of
    # three: each member ends bit-identical (rows, phenotypes, fitness, allele tables) to the same
    # population stepped alone through the same sizes, since its draws depend only on its own seed
    sched = [[300, 50, 120], [30, 400, 120], [250, 9, 20], [1, 150, 300], [90, 300, 2]]
    descs, alone = [], []
    for k in range(3):
        kw = dict(KW, seed=101 + k, max_events=1 << 16, max_mutations=1 << 13)
        pop = cg.Population(400, 1 << 13, 2, **kw)
        pop.init([200, 100, 300][k])
        for row in sched:
            pop.simulate_philox(row[k])
        alone.append(pop)
        descs.append(pop.desc)
    bt = cg.Batch(descs)
    bt.N = [200, 100, 300]
    bt.init()
    bt.run_schedule(sched)
    for k, pop in enumerate(alone):
        ib = bt.info(k)
        assert ib["device_error"] == 0 and ib["N"] == sched[-1][k]
        assert np.array_equal(bt.rows(k), pop.rows()), f"population {k}"
        assert bt.stats(k)["mean_fitness"] == pop.stats()["mean_fitness"]
        pop.close()
    bt.close()


def test_runs_on_the_callers_stream():
    torch = pytest.importorskip("torch")
    N = 1200
    a = cg.Population(N, 1 << 13, 2, **KW)
    b = cg.Population(N, 1 << 13, 2, **KW)
    for p in (a, b):
        p.init(N)
    a.run_philox(N, 8)
    s = torch.cuda.Stream()
    b.set_stream(s.cuda_stream)
    b.run_philox(N, 4)                  # captured and replayed on the caller's stream
    for _ in range(4):
        b.simulate_philox(N)
    s.synchronize()
    b.set_stream(None)                  # back to the context's own stream
    _same(_state(a), _state(b))
    for p in (a, b):
        p.close()


def test_phase_clocks_cover_every_row_and_change_no_result():
    N = 1500
    a = cg.Population(N, 1 << 13, 2, **KW)
    b = cg.Population(N, 1 << 13, 2, **KW)
    for p in (a, b):
        p.init(N)
    a.run_philox(N, 5)
    b.run_philox(N, 2)
    b.profile(True, phases=True)         # the phase-clock build of the generation kernel
    for _ in range(3):
        b.simulate_philox(N)
    ph = b.phase_clocks()
    b.profile(False)
    _same(_state(a), _state(b))
    assert ph["copy_rows"] + ph["xo_rows"] + ph["long_rows"] == 3 * 2 * N
    assert ph["copy_rows"] >= 3 * N      # the second gamete of each pair is a copy row
    assert ph["xo_rows"] > 0 and ph["xo_mask"] > 0 and 0 < ph["xo_gather"] <= ph["xo_body"]
    assert ph["warps"] > 0 and ph["warps"] % 3 == 0
    rows_cycles = sum(ph[k] for k in ("copy_setup", "copy_body", "copy_phenotype", "xo_setup", "xo_mask", "xo_body",
                                      "xo_phenotype", "long_cycles"))
    assert 0 < rows_cycles <= ph["warp_cycles"]
    b.profile(True)                      # re-enabling resets the counters; the plain build leaves them at 0
    b.simulate_philox(N)
    assert sum(b.phase_clocks().values()) == 0
    for p in (a, b):
        p.close()


def test_async_info_requests_match_synchronous_reads():
    N = 1500
    a = cg.Population(N, 1 << 13, 2, **KW)
    b = cg.Population(N, 1 << 13, 2, **KW)
    for p in (a, b):
        p.init(N)
    sync_infos = []
    for _ in range(6):
        a.simulate_philox(N)
        sync_infos.append(a.info())
    tickets = []
    for _ in range(6):
        b.simulate_philox(N)
        tickets.append(b.info_request())   # issued behind the generation, collected later
    assert [b.info_wait(t) for t in tickets] == sync_infos
    assert tickets == list(range(6))
    for _ in range(9):
        b.info_request()
    with pytest.raises(cg.ClothoError):
        b.info_wait(tickets[0])             # more than 8 requests ago: its slot was reused
    for p in (a, b):
        p.close()
    jobs = [dict(N=1200, seed=5), dict(N=900, seed=6)]
    bt = cg.Batch([cg.make_desc(j["N"], 1 << 13, 2, mu=0.05, rho=2.0, seed=j["seed"]) for j in jobs])
    bt.init()
    bt.run(3)
    t = [bt.info_request(i) for i in range(2)]
    assert [bt.info_wait(x) for x in t] == [bt.info(i) for i in range(2)]
    bt.close()


def test_a_qtlsim_configuration_runs_end_to_end():
    # a reference configuration file (string values, as Boost writes them) read into a device population
    # and run for its generations under its growth model
    from clotho_gb300 import config
    cfg = {"configuration": {
        "generations": {"size": "12"},
        "population_growth": {"name": "predefined", "params": {"sizes": ["400", "150", "600"]}},
        "mutation": {"mu": "0.05"}, "recombination": {"rho": "1.5", "sequence_bias": {"p": "0.4"}},
        "traits": {"N": "2"}, "neutral": {"p": "0.3"}, "fitness": {"name": "quadratic", "params": {"scale": "4"}},
        "random_number": {"seed": "9"}}}
    rc = config.from_reference(cfg)
    pop = rc.population()
    assert pop.info()["N"] == 400
    pop.run_philox_schedule(rc.sizes())
    i = pop.info()
    assert i["device_error"] == 0 and i["N"] == rc.sizes()[-1] and i["generation"] == 13
    assert pop.stats(16)["segregating"] > 0
    pop.close()


def _snapshot_offsets(snap):
    """Offsets of the status fields and of the free list, positions and rows inside a snapshot."""
    import struct
    header_bytes = struct.unpack_from("<I", snap, 12)[0]
    assert struct.unpack_from("<Q", snap, header_bytes - 8)[0] == len(snap)   # total_bytes ends the header
    st = 16 + 96                                                                # after magic, versions, desc
    T = struct.unpack_from("<I", snap, 16 + 8)[0]
    N, A, W = struct.unpack_from("<3I", snap, st + 8)
    free_cnt, fixed_total = struct.unpack_from("<2I", snap, st + 44)

    def r8(b):
        return (b + 7) & ~7
    o = {"rows": header_bytes}
    o["pos"] = o["rows"] + r8(2 * N * W * 8)
    o["free"] = o["pos"] + r8(A * 8) + r8(A * 4) + r8(A * 16) + r8(fixed_total * 8) + r8(fixed_total * 4) + \
        r8(fixed_total * T * 4)
    return dict(N=N, A=A, W=W, free_cnt=free_cnt), o


def test_restore_refuses_snapshots_whose_indices_leave_the_population():
    # a damaged or hand-edited snapshot is refused on the host, before any of its indices reach a
    # kernel: a free-list slot beyond the rows, a NaN allele position, a row bit at or beyond the
    # allele count
    import struct
    N = 300
    a = cg.Population(N, 4096, 2, **KW)
    a.init(N)
    a.run_philox(N, 8)
    snap = a.snapshot()
    f, o = _snapshot_offsets(snap)
    assert f["free_cnt"] > 0 and f["A"] < f["W"] * 64
    same = cg.Population(N, 4096, 2, **KW)
    bad = bytearray(snap)
    struct.pack_into("<I", bad, o["free"], f["W"] * 64 + 3)
    with pytest.raises(cg.ClothoError, match="free list"):
        same.restore(bytes(bad))
    bad = bytearray(snap)
    struct.pack_into("<d", bad, o["pos"] + 8, float("nan"))
    with pytest.raises(cg.ClothoError, match="position"):
        same.restore(bytes(bad))
    bad = bytearray(snap)
    word = o["rows"] + 8 * (f["A"] // 64)                 # row 0, the word holding slot A
    struct.pack_into("<Q", bad, word, struct.unpack_from("<Q", bad, word)[0] | (1 << (f["A"] % 64)))
    with pytest.raises(cg.ClothoError, match="beyond the allele count"):
        same.restore(bytes(bad))
    same.restore(snap)
    assert np.array_equal(same.rows(), a.rows())
    a.close()
    same.close()
