"""The drop-in `dvc` and `strain` programs against the reference's own.

tests/golden/dvc_runs.json holds end-to-end runs of the reference's `dvc`
and `strain` executables (built from its sources by oracle/build_ref.sh and
run by tests/golden/make_golden.py): the input files, point clouds, volume
layouts and the .disp / .stat / .sort.csv / strain CSV outputs. The same
inputs are written here and the drop-in programs run on them.

CPU tests: the input-file checks and their messages, the command line
modes, and the outputs written before the GPU is used (`<roi>.sort.csv`,
the .stat input echo, strain's own sort file); where the reference's own
programs are built (oracle/_ref), which input files both accept on both
sides of every limit, and strain's flag handling line for line. GPU tests:
whole runs.
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
from dvc_inputs import write_dvc_inputs  # noqa: E402

RUNS = json.load(open(os.path.join(GOLDEN, "dvc_runs.json")))


@pytest.fixture(scope="session")
def vols():
    z = np.load(os.path.join(GOLDEN, "reference_hotpath.npz"))
    return {k: (z[f"vol_{k}_ref"], z[f"vol_{k}_cor"]) for k in ("A", "B")}


@pytest.fixture(scope="session")
def bins():
    from digitalvolumecorrelation_gb300 import build
    build.build_library()
    build.build_host()
    return os.path.join(build.BIN_DIR, "dvc"), os.path.join(build.BIN_DIR, "strain")


def run(cmd, cwd):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr  # the reference's programs return 0, also on errors
    return r.stdout


def setup_run(tmp_path, run_, vols):
    d = str(tmp_path)
    write_dvc_inputs(d, run_["case"], vols, np.array(run_["points"]), run_["labels"])
    return d


def echo_part(stat):
    """The .stat input echo and point-cloud block (before the version line)."""
    return stat.split("running under dvc code version:")[0]


# ------------------------------------------------------------------ CPU ---
@pytest.mark.parametrize("k", range(len(RUNS)), ids=[r["case"]["name"] for r in RUNS])
def test_dvc_sort_file_and_echo(bins, vols, tmp_path, k):
    """<roi>.sort.csv and the .stat echo equal the reference's byte for byte
    (std::sort neighbour order with ties; starting_point handling)."""
    g = RUNS[k]
    d = setup_run(tmp_path, g, vols)
    run([bins[0], "dvc_in"], d)
    assert open(os.path.join(d, "points.roi.sort.csv")).read() == g["sort_csv"]
    assert echo_part(open(os.path.join(d, "result.stat")).read()) == echo_part(g["stat"])


BAD_INPUTS = [
    # (edit of the valid input file, message expected)
    (lambda t: t.replace("interp_type\ttricubic", "# interp_type\ttricubic"),
     "keyword 'interp_type' not found"),
    (lambda t: t.replace("num_srch_dof\t6", "num_srch_dof\t7"), "num_srch_dof contains an invalid parameter"),
    (lambda t: t.replace("ref.raw\t", "nope.raw\t"), "cannot find file: nope.raw"),
    (lambda t: t.replace("vol_wide\t40", "vol_wide\t41"), "does not match the volume description"),
    (lambda t: t + "subvol_aspect\t0.05 1 1\n", "subvol_aspect contains an invalid parameter"),
    (lambda t: t.replace("basin_radius\t1.5", "basin_radius\t3.5"), "basin_radius contains an invalid parameter"),
    (lambda t: t.replace("num_points_to_process\t0", ""), "keyword 'num_points_to_process' not found"),
    (lambda t: t.replace("subvol_thresh\toff", "subvol_thresh\ton"), "keyword 'gray_thresh_min' not found"),
    (lambda t: t.replace("vol_bit_depth\t8", "vol_bit_depth\t16"), "keyword 'vol_endian' not found"),
    (lambda t: t + "rigid_trans\t0 50 0\n", "rigid_trans contains an invalid parameter"),
]


@pytest.mark.parametrize("edit,msg", BAD_INPUTS, ids=[m for _, m in BAD_INPUTS])
def test_dvc_input_errors(bins, vols, tmp_path, edit, msg):
    d = setup_run(tmp_path, RUNS[0], vols)
    p = os.path.join(d, "dvc_in")
    text = edit(open(p).read())
    with open(p, "w") as f:
        f.write(text)
    out = run([bins[0], "dvc_in"], d)
    assert msg in out, out
    assert not os.path.exists(os.path.join(d, "result.disp"))


REF_DVC = os.path.join(ROOT, "oracle", "_ref", "dvc")


def _set_keys(text, kv):
    """The input file with each keyword's value replaced (or the keyword
    appended when the file has none)."""
    lines = text.split("\n")
    for key, val in kv.items():
        for i, l in enumerate(lines):
            if l.split("\t")[0] == key:
                lines[i] = f"{key}\t{val}\t###"
                break
        else:
            lines.insert(len(lines) - 1, f"{key}\t{val}")
    return "\n".join(lines)


# Both sides of the reference's limits
# (Core/InputRead.cpp:519-631: subvol_size and disp_max up to the smallest
# volume dimension, subvol_npts up to 50000, basin_radius up to disp_max,
# rigid_trans and starting_point within the volume's extent, subvol_aspect in
# [0.1, 10], gray thresholds within 2^vol_bit_depth, min_vol_fract in [0, 1])
_THR = {"subvol_thresh": "on", "gray_thresh_min": "10", "gray_thresh_max": "200", "min_vol_fract": "0.5"}
ACCEPTANCE = [  # (name, keyword values, accepted by both)
    ("subvol_size 40", {"subvol_size": "40"}, True),
    ("subvol_size 41", {"subvol_size": "41"}, False),
    ("subvol_npts 50000", {"subvol_npts": "50000"}, True),
    ("subvol_npts 50001", {"subvol_npts": "50001"}, False),
    ("disp_max 40", {"disp_max": "40", "basin_radius": "0"}, True),
    ("disp_max 41", {"disp_max": "41"}, False),
    ("basin_radius 3", {"basin_radius": "3"}, True),
    ("basin_radius 3.01", {"basin_radius": "3.01"}, False),
    ("basin_radius -1", {"basin_radius": "-1"}, False),
    ("num_srch_dof 3", {"num_srch_dof": "3"}, True),
    ("num_srch_dof 12", {"num_srch_dof": "12"}, True),
    ("obj_function sad", {"obj_function": "sad"}, True),
    ("obj_function nssd", {"obj_function": "nssd"}, True),
    ("obj_function ncc", {"obj_function": "ncc"}, False),
    ("interp_type nearest", {"interp_type": "nearest"}, True),
    ("interp_type cubic", {"interp_type": "cubic"}, False),
    ("subvol_geom sphere", {"subvol_geom": "sphere"}, True),
    ("subvol_geom ball", {"subvol_geom": "ball"}, False),
    ("vol_hdr_lngth 16", {"vol_hdr_lngth": "16"}, False),
    ("vol_bit_depth 12", {"vol_bit_depth": "12"}, False),
    ("rigid_trans in", {"rigid_trans": "0 -40 0"}, True),
    ("rigid_trans out", {"rigid_trans": "0 -41 0"}, False),
    ("subvol_aspect in", {"subvol_aspect": "0.1 1 10"}, True),
    ("subvol_aspect out", {"subvol_aspect": "1 10.5 1"}, False),
    ("starting_point in", {"starting_point": "20 20 40"}, True),
    ("starting_point out", {"starting_point": "20 20 41"}, False),
    ("subvol_thresh on", _THR, True),
    ("gray_thresh_max 300", dict(_THR, gray_thresh_max="300"), False),
    ("gray_thresh_max below min", dict(_THR, gray_thresh_min="100", gray_thresh_max="50"), False),
    ("min_vol_fract 1.5", dict(_THR, min_vol_fract="1.5"), False),
    ("subvol_thresh maybe", {"subvol_thresh": "maybe"}, False),
]


@pytest.mark.skipif(not os.path.exists(REF_DVC),
                    reason="the reference's dvc is built only where its sources are (oracle/build_ref.sh)")
@pytest.mark.parametrize("name,kv,expect", ACCEPTANCE, ids=[n for n, _, _ in ACCEPTANCE])
def test_dvc_accepts_what_the_reference_accepts(bins, vols, tmp_path, name, kv, expect):
    """Each edit of a valid input file, run through the drop-in `dvc` and
    through the reference's own: both accept it (read the input and the
    point cloud, then sort: `sorting finished`) or both reject it; for an
    accepted file the .stat input echo and <roi>.sort.csv are the same bytes.
    The reference searches two points of an accepted file on the CPU; the
    drop-in stops at the GPU where there is none."""
    accepted, files = {}, {}
    for tag, exe in (("drop-in", bins[0]), ("reference", REF_DVC)):
        d = os.path.join(str(tmp_path), tag)
        os.makedirs(d)
        write_dvc_inputs(d, RUNS[0]["case"], vols, np.array(RUNS[0]["points"]), RUNS[0]["labels"])
        p = os.path.join(d, "dvc_in")
        text = _set_keys(open(p).read(), dict(kv, num_points_to_process="2"))
        with open(p, "w") as f:
            f.write(text)
        r = subprocess.run([exe, "dvc_in"], cwd=d, capture_output=True, text=True, timeout=300)
        accepted[tag] = "sorting finished" in r.stdout
        if not accepted[tag]:
            assert r.returncode == 0, (tag, r.stdout[-400:], r.stderr[-400:])
        else:
            files[tag] = (echo_part(open(os.path.join(d, "result.stat")).read()),
                          open(os.path.join(d, "points.roi.sort.csv")).read())
    assert accepted == {"drop-in": expect, "reference": expect}, (name, accepted)
    if expect:  # the .stat input echo and the processing order, byte for byte
        assert files["drop-in"][0] == files["reference"][0]
        assert files["drop-in"][1] == files["reference"][1]


def _roi_variants():
    """Point-cloud files built from the first run's points, each exercising
    one of the reference's line rules (InputRead::read_point_cloud,
    Core/InputRead.cpp:632-700: an integer label, not followed by '.' or 'E',
    then three numbers; anything else skips the line; the line end is
    detected per file)."""
    P, L = RUNS[0]["points"], RUNS[0]["labels"]

    def base(fmt="{l}\t{x:g}\t{y:g}\t{z:g}", sep="\n"):
        return sep.join(fmt.format(l=l, x=p[0], y=p[1], z=p[2]) for l, p in zip(L, P)) + sep
    return {
        "header and comments": "n\tx\ty\tz\n# comment line\n\n" + base(),
        "crlf": "n x y z\r\n" + base(sep="\r\n"),
        "extra columns": base("{l} {x:g} {y:g} {z:g} 99 extra"),
        "float labels": base() + "5.0\t20\t20\t20\n7.5 21 21 21\n",
        "exponent labels": base() + "1E2 20 20 20\n7e1 21 21 21\n3e 22 22 22\n",
        "short lines": base() + "300 20 20\n301 20\n302\n",
        "scientific coordinates": base() + "400 2.05e1 1.9E1 +20.5\n401 -0 20 20.0\n",
        "tabs and spaces": base("  {l} \t {x:g}   {y:g}\t\t{z:g}  "),
        "duplicate points": base() + "500 20 20 20\n501 20 20 20\n502 19.9 20.1 20\n",
        "no final newline": base()[:-1],
        "negative labels": base("-{l}\t{x:g}\t{y:g}\t{z:g}"),
        "text in coordinates": base() + "600 20 abc 20\n601 20 20 x\n",
    }


ROI_VARIANTS = _roi_variants()


@pytest.mark.skipif(not os.path.exists(REF_DVC),
                    reason="the reference's dvc is built only where its sources are (oracle/build_ref.sh)")
@pytest.mark.parametrize("name", list(ROI_VARIANTS))
def test_dvc_reads_point_clouds_as_the_reference(bins, vols, tmp_path, name):
    """The same point-cloud file through both programs: the same points
    (count and bounding box in the .stat echo) and the same processing order
    and neighbours (<roi>.sort.csv, ties included), byte for byte."""
    files = {}
    for tag, exe in (("drop-in", bins[0]), ("reference", REF_DVC)):
        d = os.path.join(str(tmp_path), tag)
        os.makedirs(d)
        write_dvc_inputs(d, RUNS[0]["case"], vols, np.array(RUNS[0]["points"]), RUNS[0]["labels"])
        with open(os.path.join(d, "points.roi"), "w", newline="") as f:
            f.write(ROI_VARIANTS[name])
        p = os.path.join(d, "dvc_in")
        text = _set_keys(open(p).read(), {"num_points_to_process": "2", "starting_point": "20 20 20"})
        with open(p, "w") as f:
            f.write(text)
        r = subprocess.run([exe, "dvc_in"], cwd=d, capture_output=True, text=True, timeout=300)
        assert "sorting finished" in r.stdout, (tag, r.stdout[-400:])
        files[tag] = (echo_part(open(os.path.join(d, "result.stat")).read()),
                      open(os.path.join(d, "points.roi.sort.csv")).read())
    assert "Point Cloud contains" in files["reference"][0]
    assert files["drop-in"] == files["reference"]


REF_STRAIN = os.path.join(ROOT, "oracle", "_ref", "strain")
STRAIN_FLAGS = [["-sw", "30"], ["-sw", "0"], ["-sw", "5000"], ["-sw", "abc"], ["-t", "0.05"], ["-t", "5"],
                ["-t", "-1"], ["-r", "-E", "-D"], ["-A", "-xy"], ["-q", "-sw"], ["-sw", "12", "-t", "0.3", "-r"],
                ["-yz", "-zx", "-t"]]


@pytest.mark.skipif(not os.path.exists(REF_STRAIN),
                    reason="the reference's strain is built only where its sources are (oracle/build_ref.sh)")
@pytest.mark.parametrize("flags", STRAIN_FLAGS, ids=[" ".join(f) for f in STRAIN_FLAGS])
def test_strain_flags_as_the_reference(bins, tmp_path, flags):
    """strain's command line through the drop-in and the reference's own
    program: the same messages and the same settings (window, threshold,
    refill, plane, point counts), line for line up to the fit, for valid,
    clamped, malformed and unknown flags."""
    def head(out):
        lines = out.split("\n")
        for i, l in enumerate(lines):
            if l.startswith("ndisp_pts ="):
                return lines[:i + 1]
        return lines
    outs = []
    for tag, exe in (("drop-in", bins[1]), ("reference", REF_STRAIN)):
        d = os.path.join(str(tmp_path), tag)
        os.makedirs(d)
        open(os.path.join(d, "result.disp"), "w").write(RUNS[0]["disp"])
        open(os.path.join(d, "points.roi.sort.csv"), "w").write(RUNS[0]["sort_csv"])
        r = subprocess.run([exe, "result.disp", "points.roi.sort.csv"] + flags, cwd=d, capture_output=True,
                           text=True, timeout=120)
        outs.append(head(r.stdout))
    assert any(l.startswith("using strain window: ") for l in outs[1])
    assert outs[0] == outs[1]


def test_dvc_roi_rules_and_modes(bins, vols, tmp_path):
    d = setup_run(tmp_path, RUNS[0], vols)
    # a point cloud with no valid line aborts
    open(os.path.join(d, "points.roi"), "w").write("n x y z\n1.5 2 3 4\n7 8 9\n")
    out = run([bins[0], "dvc_in"], d)
    assert "No points were read" in out
    assert "Options:" in run([bins[0]], d)
    run([bins[0], "example"], d)
    ex = open(os.path.join(d, "dvc_in_example")).read()
    from digitalvolumecorrelation_gb300 import abi  # noqa: F401  (package importable)
    for kw in ("reference_filename", "vol_endian", "subvol_aspect", "num_points_to_process",
               "starting_point", "basin_radius", "min_vol_fract"):
        assert kw in ex
    run([bins[0], "manual"], d)
    assert os.path.getsize(os.path.join(d, "dvc_manual")) > 500
    assert "version" in run([bins[0], "version"], d)
    assert "Cannot find input file" in run([bins[0], "missing_file"], d)


def test_strain_cli_before_gpu(bins, tmp_path):
    d = str(tmp_path)
    assert "strain needs a .disp file" in run([bins[1]], d)
    assert "cannot find .disp file" in run([bins[1], "none.disp"], d)
    open(os.path.join(d, "bad.disp"), "w").write("1\t2\t3\t4\t0\t0.1\t0\t0\t0\n")
    assert "lacks the header" in run([bins[1], "bad.disp"], d)
    # without a sort file, strain writes its own first (std::sort order with ties)
    g = RUNS[0]["strain"]["unsorted"]
    open(os.path.join(d, "result.disp"), "w").write(RUNS[0]["disp"])
    out = run([bins[1], "result.disp", "-q"] + g["args"], d)
    assert "unused flag -q found, ignored" in out
    assert open(os.path.join(d, "result.sort.csv")).read() == g["files"]["result.sort.csv"]


# ------------------------------------------------------------------ GPU ---
def parse_disp(text):
    rows = [l.split("\t") for l in text.strip().split("\n")[1:]]
    return rows


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(len(RUNS)), ids=[r["case"]["name"] for r in RUNS])
def test_dvc_run_matches_reference(bins, vols, tmp_path, k):
    """Whole `dvc` run: rows in the reference's processing order, the same
    labels, coordinates and statuses; u, v, w within 1e-3 voxel; objmin
    within 2e-5 relative (both printed with six significant digits)."""
    g = RUNS[k]
    d = setup_run(tmp_path, g, vols)
    run([bins[0], "dvc_in"], d)
    ours = parse_disp(open(os.path.join(d, "result.disp")).read())
    ref = parse_disp(g["disp"])
    assert len(ours) == len(ref)
    for a, b in zip(ours, ref):
        assert a[:5] == b[:5], (a, b)  # n x y z status, as text
        oa, ob = float(a[5]), float(b[5])
        assert abs(oa - ob) <= 2e-5 * max(abs(ob), 1e-12) + 1e-12, (a, b)
        du = np.abs(np.array(a[6:9], float) - np.array(b[6:9], float))
        assert du.max() <= 1e-3, (a, b)
    # <out>.par: every search parameter (the reference's, from its classes
    # re-run over the program's order and neighbours)
    par_rows = [l.split("\t") for l in open(os.path.join(d, "result.par")).read().strip().split("\n")[1:]]
    par = np.array(g["par"])
    assert len(par_rows) == len(ref) and par.shape[1] == int(dict(g["case"]["keys"])["num_srch_dof"])
    for a, b, pr in zip(par_rows, ref, par):
        assert a[:5] == b[:5]
        if a[4] == "0":
            assert np.abs(np.array(a[6:], float) - pr).max() <= 1e-3, (a, pr)
    stat = open(os.path.join(d, "result.stat")).read()
    for line in g["stat"].splitlines():
        if line.startswith(("number ", "Point Cloud", "\tbounding")) or " points processed in " in line:
            key = line.split(" in ")[0] if " points processed in " in line else line
            assert key in stat, line


def close6(a, b, scale):
    """Two values each printed with six significant digits agree to within
    one unit of the sixth digit, or 1e-9 of the column's scale."""
    mag = np.maximum(np.abs(a), np.abs(b))
    unit = 10.0 ** (np.floor(np.log10(np.where(mag == 0, 1e-300, mag))) - 5)
    return np.abs(a - b) <= np.maximum(1.01 * unit, 1e-9 * scale)


@pytest.mark.gpu
@pytest.mark.parametrize("tag", ["sorted", "unsorted"])
def test_strain_run_matches_reference(bins, tmp_path, tag):
    g = RUNS[0]["strain"][tag]
    d = str(tmp_path)
    open(os.path.join(d, "result.disp"), "w").write(RUNS[0]["disp"])
    if tag == "sorted":
        open(os.path.join(d, "points.roi.sort.csv"), "w").write(RUNS[0]["sort_csv"])
    run([bins[1], "result.disp"] + g["args"], d)
    for name, text in g["files"].items():
        mine = open(os.path.join(d, name)).read()
        if name.endswith(".sort.csv"):
            assert mine == text
            continue
        a = np.array([[float(v) for v in l.split(",")] for l in mine.strip().split("\n")[1:]])
        b = np.array([[float(v) for v in l.split(",")] for l in text.strip().split("\n")[1:]])
        assert mine.split("\n")[0] == text.split("\n")[0]
        assert a.shape == b.shape
        assert np.array_equal(a[:, [0, 7]], b[:, [0, 7]]), name  # labels, points in window
        scale = np.abs(b).max(axis=0)
        ok = close6(a, b, scale[None, :])
        assert ok.all(), (name, np.argwhere(~ok)[:5], a[~ok][:5], b[~ok][:5])
