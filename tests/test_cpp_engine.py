"""The reference engine's stage sequence over the GPU adapters: tests/cpp/engine_stages_test.cpp is a
template engine in the shape of Engine<...,batched_task> (policies chosen by member typedefs, simulate()
calling them with the reference's member signatures), instantiated with the GPU policy set and a stand-in
for the reference's Boost thread pool.  It compiles and links on any host; on a GPU it must give the same
genomes as the fused engine driven by the same draws, and run with device-drawn parents."""
import os
import shutil
import subprocess

import pytest

from tests.conftest import gpu_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    from clotho_gb300 import builder
    lib = builder.build()
    exe = str(tmp_path / "engine_stages_test")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", ROOT,
                        os.path.join(ROOT, "tests", "cpp", "engine_stages_test.cpp"), "-o", exe, "-L",
                        os.path.dirname(lib), "-lclotho_gpu", "-Wl,-rpath," + os.path.dirname(lib)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_stage_sequence_compiles_against_the_adapters(tmp_path):
    assert os.access(_build(tmp_path), os.X_OK)


@pytest.mark.gpu
def test_stage_sequence_matches_the_fused_engine(tmp_path):
    if not gpu_available():
        pytest.skip("no CUDA device")
    r = subprocess.run([_build(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
