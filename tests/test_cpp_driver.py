"""The C++ policy adapters (clotho_gb300/cpp/clotho_gb300.hpp) and the
QTLSim-style driver built on them."""
import json
import os
import subprocess

import pytest

from tests.conftest import gpu_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_adapters_compile_and_driver_links():
    from clotho_gb300 import builder
    builder.build()
    assert os.access(builder.DRIVER_PATH, os.X_OK)
    # the adapter header is self-contained C++17
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-x", "c++",
                        os.path.join(ROOT, "clotho_gb300", "cpp", "clotho_gb300.hpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("staged", [0, 1])
def test_driver_runs_generations(staged):
    if not gpu_available():
        pytest.skip("no CUDA device")
    from clotho_gb300 import builder
    builder.build()
    r = subprocess.run([builder.DRIVER_PATH, "500", "30", "0.1", "1.0", "2", str(staged), "5"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.strip().splitlines()]
    status = [x for x in lines if "generation" in x]
    assert status[-1]["generation"] == 30 and status[-1]["device_error"] == 0
    assert status[-1]["alleles"] > 0
    perf = lines[-1]
    assert len(perf["performance"]["simulate"]) == 30 and len(perf["memory"]["free_count"]) == 30


@pytest.mark.gpu
def test_driver_follows_a_growth_model():
    if not gpu_available():
        pytest.skip("no CUDA device")
    from clotho_gb300 import builder
    builder.build()
    # predefined sizes (population_growth toolkit): generation k has sizes[k % 3] individuals
    r = subprocess.run([builder.DRIVER_PATH, "600", "20", "0.1", "1.0", "1", "0", "5", "predefined:300,500,400"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    status = [json.loads(x) for x in r.stdout.strip().splitlines() if '"generation"' in x]
    assert [(s["generation"], s["N"]) for s in status] == [(10, [300, 500, 400][10 % 3]), (20, [300, 500, 400][20 % 3])]
    assert all(s["device_error"] == 0 for s in status)
