"""ms export (CPU): written samples parse back to the same haplotypes, with the
segregating sites of the sample ordered by position, and the allele counts the
reference's ms tool computes (src/tools/ms/ms_allele_freq.py) follow."""
import io

import numpy as np

from clotho_gb300 import ms


def _rows(rng, S, A):
    W = ((A + 511) // 512) * 8
    bits = (rng.random((S, W * 64)) < 0.3).astype(np.uint8)
    bits[:, A:] = 0
    bits[:, 5] = 1          # fixed in the population
    bits[:, 7] = 0          # lost
    return np.packbits(bits, axis=1, bitorder="little").view(np.uint64), bits[:, :A]


def test_round_trip_of_a_sample():
    rng = np.random.default_rng(3)
    rows, bits = _rows(rng, 40, 300)
    pos = rng.random(300)
    pos[10] = pos[11]       # tie: ordered by slot
    sample = rng.choice(40, 12, replace=False)
    f = io.StringIO()
    cols = ms.write_ms(f, rows, pos, sample=sample, seeds=(1, 2, 3))
    (rep,) = ms.read_ms(f.getvalue())
    hap = bits[sample]
    cnt = hap.sum(axis=0)
    expect = [a for a in np.lexsort((np.arange(300), pos)) if 0 < cnt[a] < 12]
    assert list(cols) == expect
    assert rep["segsites"] == len(expect)
    assert np.array_equal(rep["haplotypes"], hap[:, expect])
    assert np.allclose(rep["positions"], pos[expect], atol=1e-9)
    assert 5 not in cols and 7 not in cols
    # allele counts per site, as the reference's ms tool tallies them
    assert np.array_equal(rep["haplotypes"].sum(axis=0), cnt[expect])


def test_empty_sample_and_several_replicates():
    rng = np.random.default_rng(4)
    rows, _ = _rows(rng, 6, 100)
    f = io.StringIO()
    ms.write_ms(f, rows[:1], rng.random(100))                        # one sequence: nothing segregates
    ms.write_ms(f, rows, rng.random(100), header=False)
    reps = ms.read_ms(f.getvalue())
    assert len(reps) == 2 and reps[0]["segsites"] == 0 and reps[1]["haplotypes"].shape[0] == 6
