"""Golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py
from the CPU oracle).  The CPU test pins the oracle to its recorded outputs;
the GPU test replays the recorded tapes through the C-ABI and must reproduce
rows, free list, allele and fixed tables bit for bit."""
import glob
import os

import numpy as np
import pytest

import oracle
from tests.conftest import gpu_available

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(glob.glob(os.path.join(HERE, "*.npz")))


def load(path):
    z = np.load(path)
    params = {k[len("param_"):]: z[k][0] for k in z.files if k.startswith("param_")}
    tapes = []
    for g in range(int(z["G"][0])):
        N, M = (int(v) for v in z[f"g{g}_NM"])
        tapes.append(oracle.Tape(N, M, *(z[f"g{g}_{f}"] for f in ("pairs", "swap", "ev_off", "ev_pos", "mut_seq",
                                                                   "mut_pos", "mut_eff"))))
    return z, params, tapes


def oracle_params(params):
    p = dict(params)
    out = dict(T=int(p.pop("T")), fitness=int(p.pop("fitness")), seed=int(p.pop("seed")))
    if "q1" in p:
        out["q1"] = bool(p.pop("q1"))
    out.update({k: float(v) for k, v in p.items()})
    return out


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[:-4] for c in CASES])
def test_oracle_reproduces_golden(path):
    z, params, tapes = load(path)
    orc = oracle.Oracle(threads=2, **oracle_params(params))
    orc.init(int(z["N"][0]))
    for t in tapes:
        orc.step_tape(t)
    assert np.array_equal(orc.rows(), z["rows"])
    assert np.array_equal(orc.free_list(), z["free"])
    pos, age, eff = orc.alleles()
    assert np.array_equal(pos, z["pos"]) and np.array_equal(age, z["age"]) and np.array_equal(eff, z["eff"])
    fpos, fage, feff = orc.fixed()
    assert np.array_equal(fpos, z["fixed_pos"]) and np.array_equal(feff, z["fixed_eff"])
    np.testing.assert_allclose(orc.phenotypes(), z["phenotypes"], rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(orc.fitness(), z["fitness"], rtol=1e-13, atol=1e-300)


def test_golden_covers_fixation():
    z = np.load(os.path.join(HERE, "drift_fixation.npz"))
    assert int(z["info_fixed_total"][0]) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[:-4] for c in CASES])
def test_gpu_replays_golden(path):
    if not gpu_available():
        pytest.skip("no CUDA device")
    import clotho_gb300 as cg
    z, params, tapes = load(path)
    p = oracle_params(params)
    names = {oracle.FIT_CONSTANT: "constant", oracle.FIT_GAUSSIAN: "gaussian", oracle.FIT_QUADRATIC: "quadratic",
             oracle.FIT_GAUSSIAN_VS: "gaussian_vs"}
    N = int(z["N"][0])
    cap = int(z["Ncap"][0]) if "Ncap" in z.files else N
    pop = cg.Population(cap, 4096, p["T"], fitness=names[p["fitness"]], fit_param=p.get("fit_param", 1.0),
                        mu=p["mu"], rho=p["rho"], p_neutral=p["p_neutral"], q1=p.get("q1", True),
                        max_events=1 << 14, max_mutations=1 << 12, max_fixed=1 << 14)
    pop.init(N)
    for t in tapes:
        pop.simulate(t)
    pop.check()
    assert np.array_equal(pop.rows(), z["rows"])
    assert np.array_equal(pop.free_list(), z["free"])
    pos, age, eff = pop.alleles()
    assert np.array_equal(pos, z["pos"]) and np.array_equal(age, z["age"])
    assert np.array_equal(eff.astype(np.float64), z["eff"])
    fpos, fage, feff = pop.fixed()
    assert np.array_equal(fpos, z["fixed_pos"]) and np.array_equal(fage, z["fixed_age"])
    # phenotype: the tolerance of tests/test_gpu_parity.py over G generations
    G = len(tapes)
    rows = z["rows"]
    S = rows.shape[0]
    A = eff.shape[0]
    bits = np.unpackbits(rows.view(np.uint8).reshape(S, -1), axis=1, bitorder="little")[:, :A].astype(np.float64)
    s = bits @ np.abs(eff.astype(np.float64))
    n = bits.sum(axis=1)
    worst = (((n[0::2] + n[1::2])[:, None] + 1.0) * (s[0::2] + s[1::2])).max(axis=0)
    bound = (G + 1.0) * 2.0 ** -24 * worst + 1e-30
    if not int(z["info_all_neutral"][0]):
        assert np.all(np.abs(pop.phenotypes() - z["phenotypes"]) <= bound)
