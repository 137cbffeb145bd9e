"""C ABI: the library loads and exports every entry point include/dvc_gpu.h
declares, the header is plain C (and C++), and a C program links against the
library and calls it (no GPU needed: only the version entry points run)."""
import ctypes
import os
import re
import subprocess

from digitalvolumecorrelation_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "dvc_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dvc_(?:gpu|cnn)_\w+)\s*\(", src)))


def test_library_exports_every_declared_function():
    lib = ctypes.CDLL(build.build_library())
    names = declared_functions()
    assert "dvc_gpu_process" in names and "dvc_gpu_strain" in names and "dvc_cnn_forward" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_errors_without_gpu_calls():
    lib = ctypes.CDLL(build.build_library())
    lib.dvc_gpu_abi_version.restype = ctypes.c_int
    assert lib.dvc_gpu_abi_version() == 3
    lib.dvc_gpu_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.dvc_gpu_version()


def test_metaimage_header_reader(tmp_path):
    """dvc_gpu_read_mhd is host code (no GPU call): a header with a separate
    raw file, and one with the data in the same file (LOCAL)."""
    from digitalvolumecorrelation_gb300 import engine
    sub = tmp_path / "f000"
    sub.mkdir()
    (sub / "frame.mhd").write_text(
        "ObjectType = Image\nNDims = 3\nBinaryData = True\nBinaryDataByteOrderMSB = True\n"
        "CompressedData = False\nDimSize = 150 126 127\nElementType = MET_USHORT\n"
        "HeaderSize = 12\nElementDataFile = frame.raw\n")
    info = engine.read_mhd(str(sub / "frame.mhd"))
    assert (info["nx"], info["ny"], info["nz"]) == (150, 126, 127)
    assert info["bytes_per_voxel"] == 2 and info["big_endian"] == 1 and info["header_bytes"] == 12
    assert info["data_file"] == str(sub / "frame.raw")
    head = b"NDims = 3\nDimSize = 4 3 2\nElementType = MET_UCHAR\nElementDataFile = LOCAL\n"
    (tmp_path / "local.mhd").write_bytes(head + bytes(range(24)))
    info = engine.read_mhd(str(tmp_path / "local.mhd"))
    assert info["bytes_per_voxel"] == 1 and info["header_bytes"] == len(head)
    assert info["data_file"] == str(tmp_path / "local.mhd")
    (tmp_path / "bad.mhd").write_text("NDims = 3\nDimSize = 4 3 2\nElementType = MET_FLOAT\n"
                                      "ElementDataFile = x.raw\n")
    try:
        engine.read_mhd(str(tmp_path / "bad.mhd"))
        raise AssertionError("float data accepted")
    except engine.DvcError as e:
        assert e.code == engine.E_ARG


C_PROGRAM = r"""
#include <stdio.h>
#include "dvc_gpu.h"
int main(void) {
  dvc_params p;
  (void)p;
  printf("%d %s\n", dvc_gpu_abi_version(), dvc_gpu_version());
  return dvc_gpu_abi_version() == DVC_ABI_VERSION ? 0 : 1;
}
"""


def test_header_is_plain_c_and_cxx(tmp_path):
    src = os.path.join(str(tmp_path), "use.c")
    open(src, "w").write(C_PROGRAM)
    inc = os.path.join(ROOT, "include")
    for cmd in (["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", "-I", inc, src],
                ["g++", "-std=c++11", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", "-x", "c++",
                 "-I", inc, src]):
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_c_program_links_and_calls_the_library(tmp_path):
    lib = build.build_library()
    libdir = os.path.dirname(lib)
    cudalib = os.path.join(os.path.dirname(os.path.dirname(build._nvcc())), "lib64")
    src, exe = os.path.join(str(tmp_path), "use.c"), os.path.join(str(tmp_path), "use")
    open(src, "w").write(C_PROGRAM)
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), src, "-o", exe, "-L", libdir,
                        "-ldvcgpu", "-L", cudalib, "-lcudart", f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{cudalib}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.startswith("3 ") and "sm_103a" in r.stdout, r.stdout + r.stderr
