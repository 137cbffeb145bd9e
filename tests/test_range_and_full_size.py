"""Status -1 (Range_Fail) and full-size subvolumes, pinned to the reference.

tests/golden/reference_range_large.json holds the reference's own searches
(oracle/_ref: its Core/*.cpp, run in its processing order with its neighbour
seeding) over the cases of tests/golden/recipes.py:
  * Range_Fail by each route the reference has: Gauss-Newton translating the
    subvolume out of the active box, without and after the coarse grid, for
    cube and sphere subvolumes, uint8 and uint16; and 12-dof Gauss-Newton
    whose rotation or strain grows the warped cloud's bounding box out of it
    (Core/Interpolate.cpp:474-481, Core/FloatingCloud.cpp:206-233,
    Core/Search.cpp:194-246). The coarse grid itself cannot leave the box (it
    reaches disp_max, the box disp_max + 1), and the reference has no check
    against the volume's faces: a box beyond them reads wrapped rows or an
    unfilled buffer (Core/Interpolate.cpp:177-192), not a status;
  * sphere 41 / 4000 samples / 12 dof and cube 41 / 3375 samples / 12 dof on
    a 128^3 uint16 crop;
  * a run of the reference's `dvc` program with failed points (the .disp rows
    of failed points);
and tests/golden/config1_dvc_run.json the plain-method workload (256^3 uint8,
1000 points, cube 31 / 2197 samples, znssd, tricubic, 6 dof, basin 6 /
disp_max 12) through the reference's `dvc` program.

The volumes are rendered from their recipes here and checked against the
recorded digests. Tolerances as the other parity tests: statuses identical;
u, v, w (and rotations, strains) within 1e-3 voxel; objmin within 1e-5
relative for converged points (2e-5 where both sides are read back from
six-significant-digit text).
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLDEN)
import recipes  # noqa: E402
from dvc_inputs import write_dvc_inputs  # noqa: E402

G = json.load(open(os.path.join(GOLDEN, "reference_range_large.json")))
CASES = {c["name"]: c for c in G["cases"]}
RANGE_NAMES = [c["name"] for c in recipes.RANGE_CASES]
LARGE_NAMES = [c["name"] for c in recipes.LARGE_CASES]
_vols = {}


def volumes(name):
    if name not in _vols:
        ref, cor = recipes.render(recipes.by_name(name))
        assert recipes.digest(ref, cor) == CASES[name]["digest"], "rendered volumes differ from the recorded ones"
        _vols[name] = (ref, cor)
    return _vols[name]


def compare(name, r):
    g = CASES[name]
    st = np.array(g["status"])
    np.testing.assert_array_equal(r["status"], st)
    good = st == 0
    if not good.any():
        return
    gp = np.array(g["params"])
    ndof = recipes.by_name(name)["params"]["num_srch_dof"]
    dp = np.abs(r["params"][good, :ndof] - gp[good, :ndof])
    assert dp.max() <= 1e-3, dp.max()
    assert np.all(r["params"][~good] == 0.0) and np.all(r["objmin"][~good] == 0.0)
    go = np.array(g["objmin"])[good]
    rel = np.abs(r["objmin"][good] - go) / np.abs(go)
    assert rel.max() <= 1e-5, rel.max()


# ------------------------------------------------------------------ CPU ---
def test_every_range_route_has_failed_and_the_mixed_cases_good_points():
    for name in RANGE_NAMES:
        st = np.array(CASES[name]["status"])
        assert (st == -1).sum() >= 3, name
    assert sum((np.array(CASES[n]["status"]) == 0).sum() for n in RANGE_NAMES) >= 30
    for name in LARGE_NAMES:
        assert (np.array(CASES[name]["status"]) == 0).all()


@pytest.mark.parametrize("name", RANGE_NAMES + LARGE_NAMES)
def test_oracle_vs_reference(oracle, name):
    """The FP64 restatement against the reference's recorded searches (the
    checker the GPU tests' larger cases rely on)."""
    ref, cor = volumes(name)
    g = CASES[name]
    case = recipes.by_name(name)
    o = oracle.process(recipes.params(case), ref, cor, recipes.points(case), order=np.array(g["order"], np.int32),
                       neigh=np.array(g["neigh"], np.int32))
    assert o["undefined_evals"] == 0
    np.testing.assert_array_equal(o["status"], g["status"])
    good = o["status"] == 0
    if good.any():
        assert np.abs(o["params"][good] - np.array(g["params"])[good]).max() <= 1e-9
        assert np.allclose(o["objmin"][good], np.array(g["objmin"])[good], rtol=1e-9, atol=0)


# ------------------------------------------------------------------ GPU ---
@pytest.mark.gpu
@pytest.mark.parametrize("name", RANGE_NAMES + LARGE_NAMES)
def test_search_vs_reference(gpu_lib, name):
    from digitalvolumecorrelation_gb300 import engine
    ref, cor = volumes(name)
    g = CASES[name]
    case = recipes.by_name(name)
    E = engine.Engine(recipes.params(case), ref, cor)
    r = E.process(recipes.points(case), order=np.array(g["order"], np.int32), neigh=np.array(g["neigh"], np.int32))
    compare(name, r)
    # (the engine's undefined-cell counter may be non-zero here: with a
    # rotation the range check rides on the evaluation, and the samples of an
    # evaluation whose cloud then fails it are counted before it is discarded;
    # the oracle test above shows the reference's path stays defined)
    E.close()


@pytest.mark.gpu
@pytest.mark.parametrize("cluster", [1, 8])
def test_range_fail_at_other_cluster_widths(gpu_lib, monkeypatch, cluster):
    from digitalvolumecorrelation_gb300 import engine
    monkeypatch.setenv("DVC_CLUSTER", str(cluster))
    for name in ("gn_translation_6dof", "rotation_12dof"):
        ref, cor = volumes(name)
        g = CASES[name]
        case = recipes.by_name(name)
        E = engine.Engine(recipes.params(case), ref, cor)
        r = E.process(recipes.points(case), order=np.array(g["order"], np.int32),
                      neigh=np.array(g["neigh"], np.int32))
        compare(name, r)
        E.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sphere41_4000_12dof", "cube41_3375_12dof", "strain_12dof"])
def test_rank_windows_match_reference_and_repeat_bit_for_bit(gpu_lib, monkeypatch, name):
    """The dataflow search cut into three rank windows (the first and last
    ranks at twice the body's cluster width, consecutive launches): the
    reference's statuses and parameters as before, and a second run gives the
    same bits (a point's width follows from its rank, not from timing)."""
    from digitalvolumecorrelation_gb300 import engine
    monkeypatch.setenv("DVC_WINDOWS", "5,6")
    ref, cor = volumes(name)
    g = CASES[name]
    case = recipes.by_name(name)
    E = engine.Engine(recipes.params(case), ref, cor)
    runs = []
    for _ in range(2):
        runs.append(E.process(recipes.points(case), order=np.array(g["order"], np.int32),
                              neigh=np.array(g["neigh"], np.int32)))
        n = len(g["status"])
        body = E.last_launch()["cluster"]
        assert body in (2, 4)
        assert E.last_windows() == (5, n - 6, 2 * body)
        compare(name, runs[-1])
    for k in ("status", "objmin", "params"):
        np.testing.assert_array_equal(runs[0][k], runs[1][k])
    monkeypatch.setenv("DVC_WINDOWS", "0,0")
    E.process(recipes.points(case), order=np.array(g["order"], np.int32), neigh=np.array(g["neigh"], np.int32))
    assert E.last_windows() == (n, n, E.last_launch()["cluster"])
    E.close()


@pytest.fixture(scope="module")
def dvc_bin():
    from digitalvolumecorrelation_gb300 import build
    build.build_library()
    build.build_host()
    return os.path.join(build.BIN_DIR, "dvc")


def _run_dvc(dvc_bin, run, vols, tmp_path):
    d = str(tmp_path)
    write_dvc_inputs(d, run["case"], vols, np.array(run["points"]), run["labels"])
    r = subprocess.run([dvc_bin, "dvc_in"], cwd=d, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    return d


def _disp_rows(text):
    return [l.split("\t") for l in text.strip().split("\n")[1:]]


def _compare_disp(ours, ref, stop_rule_points=0.0):
    """Rows equal as text up to the status; u, v, w within 1e-3 voxel and
    objmin within 2e-5 relative. stop_rule_points: the fraction of good
    points allowed to stop Gauss-Newton one step away from the reference,
    u within 0.02 voxel and objmin within 1e-3 relative. The reference stops
    when the last update is shorter than 0.01 voxel (Core/Search.cpp:
    220-228); where its update length lies within ~1e-4 (relative) of that
    threshold, FP32 per-sample arithmetic against its FP64 can decide the
    other way, and its slowly converging iterations end one step apart."""
    assert len(ours) == len(ref)
    bad, near = [], []
    for a, b in zip(ours, ref):
        assert a[:5] == b[:5], (a, b)  # label x y z status, as text
        oa, ob = float(a[5]), float(b[5])
        du = float(np.abs(np.array(a[6:9], float) - np.array(b[6:9], float)).max())
        rel = abs(oa - ob) / max(abs(ob), 1e-12)
        if rel > 2e-5 or du > 1e-3:
            (near if (du <= 0.02 and rel <= 1e-3) else bad).append((a[0], a[4], rel, du))
    n_good = sum(r[4] == "0" for r in ref)
    assert not bad, (len(bad), bad[:20])
    assert len(near) <= stop_rule_points * n_good, (len(near), near[:20])


def compare_par(d, run, stop_rule_points=0.0):
    """<out>.par against the reference's full parameters of the same run:
    the .disp rows' points and statuses, every num_srch_dof parameter within
    1e-3 for good points (within 0.02 for a `stop_rule_points` fraction, as
    _compare_disp), zeros for the others."""
    text = open(os.path.join(d, "result.par")).read().strip().split("\n")
    head, rows = text[0].split("\t"), [l.split("\t") for l in text[1:]]
    ref_rows = _disp_rows(run["disp"])
    par = np.array(run["par"])
    ndof = par.shape[1]
    assert head == ["n", "x", "y", "z", "status", "objmin"] + \
        ["u", "v", "w", "phi", "the", "psi", "exx", "eyy", "ezz", "exy", "eyz", "exz"][:ndof]
    assert len(rows) == len(ref_rows)
    near = 0
    for k, (a, b) in enumerate(zip(rows, ref_rows)):
        assert a[:5] == b[:5]
        got = np.array(a[6:], float)
        if a[4] == "0":
            dp = np.abs(got - par[k]).max()
            if dp > 1e-3:
                assert dp <= 0.02, (a, par[k])
                near += 1
        else:
            assert np.all(got == 0.0)
    assert near <= stop_rule_points * sum(r[4] == "0" for r in ref_rows)


def test_range_dvc_run_sort_file(dvc_bin, tmp_path):
    """CPU: the program's <roi>.sort.csv is the reference's byte for byte
    (it is written before the GPU is used)."""
    run = G["dvc_run"]
    d = _run_dvc(dvc_bin, run, {run["case"]["volumes"]: volumes(run["case"]["volumes"])}, tmp_path)
    assert open(os.path.join(d, "points.roi.sort.csv")).read() == run["sort_csv"]


@pytest.mark.gpu
def test_range_dvc_run_matches_reference(dvc_bin, tmp_path):
    """The drop-in `dvc` over a case with failed points: the same rows; a
    failed row carries objmin 0 and zero displacements, as the reference's
    final rewrite of the file from its stored results (Core/dvc.cpp:314-320)."""
    run = G["dvc_run"]
    d = _run_dvc(dvc_bin, run, {run["case"]["volumes"]: volumes(run["case"]["volumes"])}, tmp_path)
    ours = _disp_rows(open(os.path.join(d, "result.disp")).read())
    ref = _disp_rows(run["disp"])
    assert sum(r[4] == "-1" for r in ref) >= 3 and sum(r[4] == "0" for r in ref) >= 3
    _compare_disp(ours, ref)
    compare_par(d, run)
    stat = open(os.path.join(d, "result.stat")).read()
    for key in ("number successful", "number range fail"):
        line = [l for l in run["stat"].splitlines() if l.startswith(key)][0]
        assert line in stat


C1 = json.load(open(os.path.join(GOLDEN, "config1_dvc_run.json")))


@pytest.fixture(scope="module")
def config1_vols():
    W, ref, cor = recipes.config1_volumes()
    assert recipes.digest(ref, cor) == C1["digest"], "rendered volumes differ from the recorded ones"
    return {"config1": (ref, cor)}


def test_config1_sort_file(dvc_bin, config1_vols, tmp_path):
    """CPU: order and 75 nearest neighbours of the 1000-point grid, as the
    reference's `dvc` wrote them."""
    d = _run_dvc(dvc_bin, C1, config1_vols, tmp_path)
    assert open(os.path.join(d, "points.roi.sort.csv")).read() == C1["sort_csv"]


@pytest.mark.gpu
def test_config1_dvc_run_matches_reference(dvc_bin, config1_vols, tmp_path):
    d = _run_dvc(dvc_bin, C1, config1_vols, tmp_path)
    # one point of the 1000 has its reference update at 1.00013 x the stop
    # threshold (0.01 voxel): allow 0.5% such points
    _compare_disp(_disp_rows(open(os.path.join(d, "result.disp")).read()), _disp_rows(C1["disp"]),
                  stop_rule_points=0.005)
    compare_par(d, C1, stop_rule_points=0.005)
