"""The binding a maintainer of the reference adds to its `dvc` program
(digitalvolumecorrelation_gb300/reference_binding/dvc_gpu_binding.cpp: the
run's points searched through the C ABI, data.results filled as the
reference's catch blocks fill them) compiles against the reference's own
headers: every RunControl, DataCloud and result field it uses exists with the
type it assumes. Runs where the reference sources are present."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BINDING = os.path.join(ROOT, "digitalvolumecorrelation_gb300", "reference_binding", "dvc_gpu_binding.cpp")


def _compile(src):
    from oracle.oracle import reference_dir
    ref = reference_dir()
    if not ref:
        pytest.skip("the reference sources are not on this machine")
    o = os.path.join(ROOT, "oracle")
    return subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-I", os.path.join(o, "ref_include"),
                           "-I", os.path.join(o, "eigen_shim"), "-I", os.path.join(ref, "Core"),
                           "-I", os.path.join(ROOT, "include"), src], capture_output=True, text=True)


def test_binding_compiles_against_the_reference_headers():
    r = _compile(BINDING)
    assert r.returncode == 0, r.stderr


def test_binding_check_sees_a_wrong_field(tmp_path):
    """The check is not vacuous: the same file with one RunControl field
    misspelt does not compile."""
    bad = os.path.join(str(tmp_path), "bad.cpp")
    src = open(BINDING).read()
    assert "run.obj_fcn" in src
    open(bad, "w").write(src.replace("run.obj_fcn", "run.obj_fcn_misspelt"))
    assert _compile(bad).returncode != 0
