"""pytest configuration: the `gpu` marker and shared helpers.

Tests marked gpu need a CUDA device and the sm_103a build of libclotho_gpu.so;
everything else runs on the CPU (oracle, golden vectors, host logic, ABI
symbol checks)."""
import os
import sys


ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available() -> bool:
    try:
        import ctypes
        rt = None
        for name in ("libcudart.so", "libcudart.so.13", "libcuda.so.1"):
            try:
                rt = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if rt is None:
            return False
        if hasattr(rt, "cudaGetDeviceCount"):
            n = ctypes.c_int(0)
            return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
        n = ctypes.c_int(0)
        return rt.cuInit(0) == 0 and rt.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False
