"""The C++ adapters read QTLSim configuration trees: tests/cpp/config_tree_test.cpp
compiles params_from / growth_from / generations_from against a stand-in for
boost::property_tree::ptree (Boost is not needed) and checks keys and defaults."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_configuration_tree_reading(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "config_tree_test")
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-I", ROOT, os.path.join(ROOT, "tests", "cpp",
                    "config_tree_test.cpp"), "-o", exe], check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
