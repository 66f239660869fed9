"""Host-side logic: tape container, neutral tape writer, workload set-up."""
import io

import numpy as np

from clotho_gb300 import tape as tp
from clotho_gb300 import workloads as wl


def test_tape_roundtrip():
    rng = np.random.default_rng(0)
    tapes = [tp.neutral_tape(rng, 50, 0.2, 1.0, T=3, p_neutral=0.3) for _ in range(3)]
    buf = io.BytesIO()
    tp.save_tapes(buf, tapes)
    buf.seek(0)
    back = tp.load_tapes(buf)
    assert len(back) == 3
    for a, b in zip(tapes, back):
        assert (a.N, a.M) == (b.N, b.M)
        for f in ("pairs", "swap", "ev_off", "ev_pos", "mut_seq", "mut_pos", "mut_eff"):
            assert np.array_equal(getattr(a, f), getattr(b, f))


def test_neutral_tape_shapes_and_laws():
    rng = np.random.default_rng(1)
    N, mu, rho, T = 20000, 0.05, 2.0, 2
    t = tp.neutral_tape(rng, N, mu, rho, T=T, p_neutral=0.5)
    S = 2 * N
    assert t.pairs.shape == (S,) and t.pairs.max() < N
    assert t.ev_off.shape == (S + 1,) and t.ev_off[0] == 0 and np.all(np.diff(t.ev_off.astype(np.int64)) >= 0)
    assert len(t.ev_pos) == t.ev_off[-1]
    assert abs(t.ev_off[-1] / S - rho) < 0.05
    assert abs(t.M / (S * mu) - 1) < 0.1
    assert t.mut_eff.shape == (t.M * T,)
    assert abs((t.mut_eff == 0).mean() - 0.5) < 0.05
    assert np.all((t.ev_pos >= 0) & (t.ev_pos < 1)) and np.all(t.mut_seq < S)


def test_neutral_spectrum_thresholds():
    rng = np.random.default_rng(2)
    S, A = 20000, 5000
    thr = wl.neutral_spectrum_thresholds(rng, S, A)
    f = thr.astype(np.float64) / 2 ** 32
    # 1/i spectrum: mean carrier fraction ~ 1/H_{S-1}
    H = np.sum(1.0 / np.arange(1, S))
    assert abs(f.mean() * H - 1.0) < 0.15
    assert f.min() > 0 and f.max() < 1


def test_seeded_start_shapes():
    pos, eff, thr = wl.seeded_start(wl.LARGE_N, N=1000)
    A = wl.LARGE_N.seeded_alleles
    assert pos.shape == (A,) and eff.shape == (A * wl.LARGE_N.T,) and thr.shape == (A,)
