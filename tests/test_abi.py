"""C ABI: the library loads and exports every entry point include/dvc_gpu.h
declares (no GPU needed: nothing is called)."""
import ctypes
import os
import re

from digitalvolumecorrelation_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "dvc_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dvc_gpu_\w+)\s*\(", src)))


def test_library_exports_every_declared_function():
    lib = ctypes.CDLL(build.build_library())
    names = declared_functions()
    assert "dvc_gpu_process" in names and "dvc_gpu_strain" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_errors_without_gpu_calls():
    lib = ctypes.CDLL(build.build_library())
    lib.dvc_gpu_abi_version.restype = ctypes.c_int
    assert lib.dvc_gpu_abi_version() == 1
    lib.dvc_gpu_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.dvc_gpu_version()
