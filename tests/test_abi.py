"""The C-ABI library loads and exports every entry point that include/*.h
declares (no compute call: this runs without a GPU)."""
import ctypes
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(clotho_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from clotho_gb300 import builder
    path = builder.build()
    lib = ctypes.CDLL(path)
    headers = glob.glob(os.path.join(ROOT, "include", "*.h"))
    assert headers
    names = [n for h in headers for n in declared(h)]
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    from clotho_gb300 import capi
    names = declared(os.path.join(ROOT, "include", "clotho_gpu.h"))
    assert set(names) <= set(capi.SIGNATURES), set(names) - set(capi.SIGNATURES)


def test_library_is_sm103a_only():
    # the build targets sm_103a alone (no PTX for other architectures)
    from clotho_gb300 import builder
    assert builder.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_footprint_query_needs_no_gpu():
    from clotho_gb300 import capi
    L = capi.load()
    d = capi.Desc(1000, 4096, 2, 1000, 100, 100, 0, 1, 1.0, 0.01, 0.01, 0.5, 0.5, 0.0, 1.0, 1)
    b = L.clotho_footprint_for(ctypes.byref(d))
    # two populations of 2000 rows x 64 words dominate
    assert b >= 2 * 2000 * 64 * 8


def test_oracle_exports_its_header():
    import oracle
    lib = ctypes.CDLL(oracle.build())
    text = open(os.path.join(ROOT, "oracle", "clotho_oracle.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = sorted(set(re.findall(r"\b(orc_[a-z_0-9]+)\s*\(", text)))
    assert names and all(hasattr(lib, n) for n in names)
