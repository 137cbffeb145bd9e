"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run here, where the reference sources exist:

    python tests/golden/make_golden.py

It builds the reference's own Core/*.cpp (oracle/build_ref.sh) and records,
on small seeded synthetic volumes, what the reference computes:
  * interpolation values (Interpolate::nearest / tri_lin / tri_cub_Lek),
  * objective values and residuals (obj_SAD .. obj_ZNSSD),
  * whole-search results (Search::process_point over a point grid, in the
    reference's order with its neighbour seeding, sphere test seed 1),
  * strain-program CSV outputs (the reference `strain` executable),
  * the 10-nearest-neighbour table of the reference's own DataCloud test
    (Core/tests/test_DataCloud.cpp:129-139 over Core/tests/grid_input.roi),
  * end-to-end runs of the reference's `dvc` and `strain` programs
    (input file, point cloud and raw volumes -> .disp, .stat, .sort.csv,
    strain CSVs); `--dvc-runs` regenerates only these;
  * `--range-large`: the searches of tests/golden/recipes.py (Range_Fail by
    each route, full-size subvolumes on a 128^3 crop) and a `dvc` program run
    with failed points -> reference_range_large.json (volumes rendered from
    their recipes at test time, checked by digest);
  * `--config1`: the plain-method workload (256^3 uint8, 1000 points, cube
    31, 6 dof) end to end through the reference's `dvc` -> config1_dvc_run.json;
  * `--alt-search`: the search stages the reference's source holds but never
    selects (random_global with its clock fixed, Nelder-Mead through
    look_with(amoeba)) on the small volumes -> reference_alt_search.json.
Machines without the reference sources run the tests from these files.
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from digitalvolumecorrelation_gb300 import synth  # noqa: E402
from digitalvolumecorrelation_gb300.abi import make_params  # noqa: E402
from oracle.oracle import REF_SO, Oracle, Reference, build_reference, reference_dir  # noqa: E402

sys.path.insert(0, HERE)
import recipes  # noqa: E402
from dvc_inputs import write_dvc_inputs  # noqa: E402

SHAPE = (40, 40, 40)

# search configurations run by the reference (volume set, params)
SEARCH_CASES = [
    ("A", dict(subvol_geom="cube", subvol_size=11, subvol_npts=300, obj_function="znssd",
               interp_type="tricubic", num_srch_dof=6, disp_max=3, basin_radius=1.5)),
    ("A", dict(subvol_geom="sphere", subvol_size=11, subvol_npts=300, obj_function="znssd",
               interp_type="tricubic", num_srch_dof=12, disp_max=3, basin_radius=1.0)),
    ("A", dict(subvol_geom="cube", subvol_size=9, subvol_npts=200, obj_function="ssd",
               interp_type="tricubic", num_srch_dof=3, disp_max=2, basin_radius=0.0)),
    ("A", dict(subvol_geom="cube", subvol_size=9, subvol_npts=125, obj_function="zssd",
               interp_type="trilinear", num_srch_dof=6, disp_max=2, basin_radius=1.0)),
    ("A", dict(subvol_geom="sphere", subvol_size=11, subvol_npts=250, obj_function="nssd",
               interp_type="tricubic", num_srch_dof=6, disp_max=2, basin_radius=2.0)),
    ("A", dict(subvol_geom="cube", subvol_size=11, subvol_npts=343, obj_function="sad",
               interp_type="nearest", num_srch_dof=3, disp_max=2, basin_radius=1.0)),
    ("B", dict(subvol_geom="sphere", subvol_size=13, subvol_npts=400, obj_function="znssd",
               interp_type="tricubic", num_srch_dof=12, disp_max=3, basin_radius=1.5)),
    ("B", dict(subvol_geom="cube", subvol_size=11, subvol_npts=343, obj_function="znssd",
               interp_type="tricubic", num_srch_dof=6, disp_max=3, basin_radius=3.0)),
]


def volumes():
    bA = synth.blobs(SHAPE, 90, seed=11)
    affA = synth.Affine(t=(1.3, -0.7, 0.4), E=((0.005, 0, 0), (0, 0.005, 0), (0, 0, 0.005)),
                        c=(20.0, 20.0, 20.0))
    A_ref = synth.render(SHAPE, bA, noise_sigma=2.0, noise_seed=12)
    A_cor = synth.render(SHAPE, bA, deform=affA, noise_sigma=2.0, noise_seed=13)
    bB = synth.blobs(SHAPE, 110, amp=(2000.0, 60000.0), seed=21)
    sinB = synth.Sinusoid(A=1.2, L=48.0)
    B_ref = synth.render(SHAPE, bB, noise_sigma=150.0, noise_seed=22, dtype=np.uint16)
    B_cor = synth.render(SHAPE, bB, deform=sinB, noise_sigma=150.0, noise_seed=23, dtype=np.uint16)
    return {"A": (A_ref, A_cor), "B": (B_ref, B_cor)}


def datacloud_golden():
    ref_dir = reference_dir()
    roi = os.path.join(ref_dir, "Core", "tests", "grid_input.roi")
    src = open(os.path.join(ref_dir, "Core", "tests", "test_DataCloud.cpp")).read()
    block = re.search(r"std::vector<int> row = \{(.*?)\};", src, re.S).group(1)
    table = [int(v) for v in re.findall(r"-?\d+", block)]
    pts = []
    for line in open(roi):
        f = line.split()
        if len(f) >= 4:
            pts.append([float(f[1]), float(f[2]), float(f[3])])
    return dict(points=pts, knn10=np.array(table).reshape(10, 10).tolist(),
                source="Core/tests/test_DataCloud.cpp:129-139, Core/tests/grid_input.roi")


def strain_golden(tmp):
    """Run the reference `strain` program on a synthetic .disp/.sort.csv."""
    rng = np.random.default_rng(5)
    g = synth.grid_points((6, 6, 6), 10.0, (60.0, 70.0, 80.0))
    n = len(g)
    X = g - np.array([60.0, 70.0, 80.0])
    disp = (np.array([0.3, -0.2, 0.1]) + X @ np.array([[0.004, 0.001, 0.0], [0.0, -0.003, 0.002],
                                                          [0.001, 0.0, 0.002]]).T
            + 1e-4 * X ** 2 + rng.normal(0, 0.01, (n, 3)))
    status = np.zeros(n, np.int32)
    status[rng.choice(n, 12, replace=False)] = -1
    objmin = rng.uniform(0.001, 0.2, n)
    disp[status != 0] = 0.0
    objmin[status != 0] = 0.0
    O = Oracle()
    order, neigh = O.order_neighbours(g)
    out = {}
    for name, pts, args in [("vol", g, ["-sw", "20", "-A"]),
                            ("vol_t", g, ["-sw", "15", "-t", "0.1", "-r", "-A"]),
                            ("planar", g * np.array([1, 1, 0]) + np.array([0, 0, 55.0]), ["-sw", "12", "-A"])]:
        d = os.path.join(tmp, name)
        os.makedirs(d, exist_ok=True)
        base = os.path.join(d, "run")
        with open(base + ".disp", "w") as f:
            f.write("n\tx\ty\tz\tstatus\tobjmin\tu\tv\tw\n")
            for i in range(n):
                f.write(f"{i + 1}\t{pts[i, 0]:.6g}\t{pts[i, 1]:.6g}\t{pts[i, 2]:.6g}\t{status[i]}\t"
                        f"{objmin[i]:.6g}\t{disp[i, 0]:.6f}\t{disp[i, 1]:.6f}\t{disp[i, 2]:.6f}\n")
        _, nb = O.order_neighbours(pts)
        with open(base + ".sort.csv", "w") as f:
            for row in nb:
                f.write(",".join(str(v) for v in row) + "\n")
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "strain"), base + ".disp",
                        base + ".sort.csv"] + args, cwd=d, check=True, capture_output=True)
        # the values exactly as the reference read them back from the text files
        rows = [l.split() for l in open(base + ".disp")][1:]
        pts = np.array([[float(r[1]), float(r[2]), float(r[3])] for r in rows])
        objmin = np.array([float(r[5]) for r in rows])
        disp = np.array([[float(r[6]), float(r[7]), float(r[8])] for r in rows])
        res = {}
        for kind in ("Lstr", "Estr", "dgrd"):
            fn = [x for x in os.listdir(d) if x.endswith(f".{kind}.csv")][0]
            rows = [l.strip().split(",") for l in open(os.path.join(d, fn))][1:]
            res[kind] = np.array([[float(v) for v in r] for r in rows])
        out[name] = dict(points=pts, status=status, objmin=objmin, disp=disp, neigh=nb,
                         args=args, **res)
    return out


# end-to-end runs of the reference's own `dvc` and `strain` programs
# (cube subvolumes: the reference's normal runs seed sphere samples from the
# clock). Inputs are written from the fixture volumes at test time.
DVC_RUNS = [
    dict(name="u8_nostart", volumes="A", header=0, endian="little",
         roi_extra="n\tx\ty\tz\n# comment line\n7.5 1 2 3\n",
         keys=[("subvol_geom", "cube"), ("subvol_size", "11"), ("subvol_npts", "300"),
               ("subvol_thresh", "off"), ("disp_max", "3"), ("num_srch_dof", "6"),
               ("obj_function", "znssd"), ("interp_type", "tricubic"), ("basin_radius", "1.5"),
               ("num_points_to_process", "0")]),
    dict(name="u16be_start", volumes="B", header=32, endian="big", roi_extra="",
         keys=[("subvol_geom", "cube"), ("subvol_size", "11"), ("subvol_npts", "343"),
               ("subvol_thresh", "off"), ("disp_max", "3"), ("num_srch_dof", "12"),
               ("obj_function", "zssd"), ("interp_type", "tricubic"), ("basin_radius", "0.0"),
               ("rigid_trans", "0.5 -0.3 0.2"), ("starting_point", "21.0 19.0 20.0"),
               ("num_points_to_process", "20")]),
]


def params_from_keys(shape, bpv, keys):
    """dvc_params of a `dvc` input file's search keys."""
    kw = {}
    for k, v in keys:
        if k in ("subvol_geom", "obj_function", "interp_type"):
            kw[k] = v
        elif k in ("subvol_size", "subvol_npts", "disp_max", "num_srch_dof"):
            kw[k] = int(v)
        elif k == "basin_radius":
            kw[k] = float(v)
        elif k in ("rigid_trans", "subvol_aspect"):
            kw[k] = tuple(float(x) for x in v.split())
    return make_params(shape, bytes_per_voxel=bpv, **kw)


def reference_full_params(d, case, vols, pts):
    """Every search parameter of a finished reference `dvc` run (its .disp
    keeps u, v, w only): the reference's own Search::process_point run again
    through its classes with the run's processing order (the .disp row order)
    and neighbour lists (its .sort.csv). Rows in .disp order; u, v, w checked
    against the .disp text."""
    vref, vcor = vols[case["volumes"]]
    shape = vref.shape[::-1]
    p = params_from_keys(shape, vref.dtype.itemsize, case["keys"])
    rows = [l.split("\t") for l in open(os.path.join(d, "result.disp")).read().strip().split("\n")[1:]]
    neigh = np.array([[int(v) for v in l.split(",")]
                      for l in open(os.path.join(d, "points.roi.sort.csv")).read().strip().split("\n")], np.int32)
    labels_file = [int(l.split()[0]) for l in open(os.path.join(d, "points.roi")) if _roi_line(l)]
    where = {lab: i for i, lab in enumerate(labels_file)}
    order = np.array([where[int(r[0])] for r in rows], np.int32)
    r = Reference().process(p, vref, cor=vcor, points=pts, order=order, neigh=neigh)
    par = r["params"][order]
    uvw = np.array([[float(v) for v in row[6:9]] for row in rows])
    assert np.abs(par[:, :3] - uvw).max() <= 5.1e-7, "re-run differs from the program's .disp"
    assert (r["status"][order] == np.array([int(row[4]) for row in rows])).all()
    return par[:, :p.num_srch_dof].tolist()


def _roi_line(line):
    """A point-cloud line the reference keeps: an integer label first (the
    lines written here are either that or the skipped header/comment)."""
    f = line.split()
    if len(f) < 4:
        return False
    try:
        int(f[0])
        float(f[1]), float(f[2]), float(f[3])
    except ValueError:
        return False
    return "." not in f[0] and "e" not in f[0].lower()


def dvc_runs_golden(tmp, vols):
    rng = np.random.default_rng(9)
    pts = synth.grid_points((3, 3, 3), 5.0, (20.0, 20.0, 20.0)) + rng.uniform(-0.4, 0.4, (27, 3)).round(2)
    labels = rng.permutation(np.arange(101, 128))
    runs = []
    for case in DVC_RUNS:
        d = os.path.join(tmp, case["name"])
        os.makedirs(d, exist_ok=True)
        write_dvc_inputs(d, case, vols, pts, labels)
        r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "dvc"), "dvc_in"], cwd=d,
                           capture_output=True, text=True, env=dict(os.environ, OMP_NUM_THREADS="4"))
        assert r.returncode == 0, r.stdout + r.stderr
        out = dict(case=case, points=pts.tolist(), labels=labels.tolist(),
                   disp=open(os.path.join(d, "result.disp")).read(),
                   sort_csv=open(os.path.join(d, "points.roi.sort.csv")).read(),
                   stat=open(os.path.join(d, "result.stat")).read(),
                   par=reference_full_params(d, case, vols, pts))
        if case["name"] == "u8_nostart":
            # the reference `strain` on this run's outputs: with the sort file
            # and without it (strain then writes its own)
            st = {}
            for tag, extra in (("sorted", ["points.roi.sort.csv"]), ("unsorted", [])):
                sd = os.path.join(d, tag)
                os.makedirs(sd, exist_ok=True)
                open(os.path.join(sd, "result.disp"), "w").write(out["disp"])
                if extra:
                    open(os.path.join(sd, extra[0]), "w").write(out["sort_csv"])
                args = ["-sw", "12", "-A"] if tag == "sorted" else ["-t", "0.5", "-r", "-E"]
                r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "strain"), "result.disp"]
                                   + extra + args, cwd=sd, capture_output=True, text=True)
                assert r.returncode == 0, r.stdout + r.stderr
                st[tag] = dict(args=extra + args,
                               files={f: open(os.path.join(sd, f)).read() for f in sorted(os.listdir(sd))
                                      if f.endswith(".csv") and f != "points.roi.sort.csv"})
            out["strain"] = st
        runs.append(out)
    return runs


def run_reference_dvc(d, env_threads="8"):
    r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "dvc"), "dvc_in"], cwd=d,
                       capture_output=True, text=True, env=dict(os.environ, OMP_NUM_THREADS=env_threads))
    assert r.returncode == 0, r.stdout + r.stderr
    return dict(disp=open(os.path.join(d, "result.disp")).read(),
                sort_csv=open(os.path.join(d, "points.roi.sort.csv")).read(),
                stat=open(os.path.join(d, "result.stat")).read())


def range_large_golden(tmp):
    """Reference searches of recipes.RANGE_CASES and LARGE_CASES (the
    reference's own Search::process_point in its order with its neighbour
    seeding, sphere test seed 1), plus one `dvc` program run with failed
    points. A case is recorded only if the FP64 oracle agrees on every status
    and none of its evaluations fell in the box's last cell plane (where the
    reference reads past its arrays and its result is undefined)."""
    R = Reference()
    O = Oracle()
    out = dict(cases=[])
    for case in recipes.RANGE_CASES + recipes.LARGE_CASES:
        ref, cor = recipes.render(case)
        pts = recipes.points(case)
        p = recipes.params(case)
        order, neigh = R.order_neighbours(pts)
        r = R.process(p, ref, cor, points=pts, order=order, neigh=neigh)
        o = O.process(p, ref, cor, pts, order=order, neigh=neigh)
        assert (o["status"] == r["status"]).all(), case["name"]
        assert o["undefined_evals"] == 0, (case["name"], o["undefined_evals"])
        out["cases"].append(dict(name=case["name"], digest=recipes.digest(ref, cor),
                                 order=order.tolist(), neigh=neigh.tolist(),
                                 status=r["status"].tolist(), objmin=r["objmin"].tolist(),
                                 params=r["params"].tolist()))
        c = dict(zip(*np.unique(r["status"], return_counts=True)))
        print(case["name"], {int(k): int(v) for k, v in c.items()})
    # the `dvc` program over a case with failed points (cube: the program's
    # sphere samples are clock-seeded)
    spec = recipes.RANGE_DVC_RUN
    case = recipes.by_name(spec["case"])
    ref, cor = recipes.render(case)
    pts = recipes.points(case)
    labels = np.random.default_rng(spec["labels_seed"]).permutation(np.arange(1, len(pts) + 1))
    keys = [(k, str(v)) for k, v in case["params"].items()] + [("subvol_thresh", "off"),
                                                               ("num_points_to_process", "0")]
    run_case = dict(name="range_run", volumes=case["name"], header=spec["header"], endian=spec["endian"],
                    roi_extra=spec["roi_extra"], keys=keys)
    d = os.path.join(tmp, "range_run")
    os.makedirs(d, exist_ok=True)
    write_dvc_inputs(d, run_case, {case["name"]: (ref, cor)}, pts, labels)
    res = run_reference_dvc(d)
    res["par"] = reference_full_params(d, run_case, {case["name"]: (ref, cor)}, pts)
    out["dvc_run"] = dict(case=run_case, digest=recipes.digest(ref, cor), points=pts.tolist(),
                          labels=labels.tolist(), **res)
    return out


# the alternative search stages (volume set, params): Nelder-Mead after the
# grid, random_global before Gauss-Newton or Nelder-Mead, 3 / 6 / 12 dof
ALT_CASES = [
    ("A", dict(subvol_geom="cube", subvol_size=11, subvol_npts=343, obj_function="znssd", num_srch_dof=3,
               disp_max=3, basin_radius=1.5, refine_method="nelder_mead")),
    ("A", dict(subvol_geom="cube", subvol_size=11, subvol_npts=343, obj_function="znssd", num_srch_dof=6,
               disp_max=3, basin_radius=1.5, refine_method="nelder_mead")),
    ("B", dict(subvol_geom="sphere", subvol_size=13, subvol_npts=400, obj_function="ssd", num_srch_dof=6,
               disp_max=3, basin_radius=0.0, refine_method="nelder_mead")),
    ("A", dict(subvol_geom="cube", subvol_size=11, subvol_npts=343, obj_function="znssd", num_srch_dof=6,
               disp_max=3, basin_radius=1.5, coarse_method="random", coarse_seed=20240613)),
    ("B", dict(subvol_geom="cube", subvol_size=11, subvol_npts=343, obj_function="zssd", num_srch_dof=3,
               disp_max=3, basin_radius=1.0, coarse_method="random", coarse_seed=7,
               refine_method="nelder_mead")),
    ("A", dict(subvol_geom="cube", subvol_size=11, subvol_npts=343, obj_function="znssd", num_srch_dof=12,
               disp_max=3, basin_radius=1.5, refine_method="nelder_mead")),
]


def alt_search_golden():
    z = np.load(os.path.join(HERE, "reference_hotpath.npz"))
    R = Reference()
    O = Oracle()
    pts, order, neigh = z["search_points"], z["search_order"], z["search_neigh"]
    out = []
    for vs, kw in ALT_CASES:
        vref, vcor = z[f"vol_{vs}_ref"], z[f"vol_{vs}_cor"]
        p = make_params(SHAPE, bytes_per_voxel=vref.dtype.itemsize, interp_type="tricubic", **kw)
        r = R.process_stages(p, vref, vcor, pts, order, neigh)
        o = O.process(p, vref, vcor, pts, order=order, neigh=neigh)
        assert (o["status"] == r["status"]).all() and np.abs(o["params"] - r["params"]).max() == 0.0
        out.append(dict(volumes=vs, params=kw, status=r["status"].tolist(), objmin=r["objmin"].tolist(),
                        params_out=r["params"].tolist(), nfunc=o["gn_iters"].tolist()))
        print(vs, kw, {int(k): int(v) for k, v in zip(*np.unique(r["status"], return_counts=True))})
    return out


def config1_golden(tmp):
    """The plain-method workload through the reference's `dvc` program."""
    W, ref, cor = recipes.config1_volumes()
    pts = W.points
    labels = np.arange(1, len(pts) + 1)
    kw = W.params_kw
    keys = [(k, str(v)) for k, v in kw.items()] + [("subvol_thresh", "off"), ("num_points_to_process", "0")]
    run_case = dict(name="config1", volumes="config1", header=0, endian="little", roi_extra="", keys=keys)
    d = os.path.join(tmp, "config1")
    os.makedirs(d, exist_ok=True)
    write_dvc_inputs(d, run_case, {"config1": (ref, cor)}, pts, labels)
    res = run_reference_dvc(d)
    res["par"] = reference_full_params(d, run_case, {"config1": (ref, cor)}, pts)
    return dict(case=run_case, digest=recipes.digest(ref, cor), points=pts.tolist(), labels=labels.tolist(),
                **res)


def main():
    if "--alt-search" in sys.argv:
        if not os.path.exists(REF_SO) and build_reference() is None:
            raise SystemExit("reference sources not available")
        with open(os.path.join(HERE, "reference_alt_search.json"), "w") as f:
            json.dump(alt_search_golden(), f)
        print("reference_alt_search.json written")
        return
    if "--range-large" in sys.argv or "--config1" in sys.argv:
        if not os.path.exists(REF_SO) or not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "dvc")):
            if build_reference() is None:
                raise SystemExit("reference sources not available")
        with tempfile.TemporaryDirectory() as tmp:
            if "--range-large" in sys.argv:
                g = range_large_golden(tmp)
                with open(os.path.join(HERE, "reference_range_large.json"), "w") as f:
                    json.dump(g, f)
                print("reference_range_large.json written")
            if "--config1" in sys.argv:
                g = config1_golden(tmp)
                with open(os.path.join(HERE, "config1_dvc_run.json"), "w") as f:
                    json.dump(g, f)
                print("config1_dvc_run.json written")
        return
    if "--dvc-runs" in sys.argv:  # only the end-to-end program runs
        if not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "dvc")):
            if build_reference() is None:
                raise SystemExit("reference sources not available")
        z = np.load(os.path.join(HERE, "reference_hotpath.npz"))
        vols = {k: (z[f"vol_{k}_ref"], z[f"vol_{k}_cor"]) for k in ("A", "B")}
        with tempfile.TemporaryDirectory() as tmp:
            runs = dvc_runs_golden(tmp, vols)
        with open(os.path.join(HERE, "dvc_runs.json"), "w") as f:
            json.dump(runs, f, indent=1)
        print("dvc_runs.json written")
        return
    if not os.path.exists(REF_SO):
        if build_reference() is None:
            raise SystemExit("reference sources not available")
    R = Reference()
    vols = volumes()
    rng = np.random.default_rng(7)
    out = {}
    # interpolation
    for vs, (vref, vcor) in vols.items():
        bpv = 1 if vref.dtype == np.uint8 else 2
        p = make_params(SHAPE, bytes_per_voxel=bpv, subvol_size=11, subvol_npts=300, disp_max=3)
        center = np.array([19.6, 20.3, 20.45])
        pts = center + rng.uniform(-9.4, 9.4, (400, 3))
        # the box's last cell plane (index n-1) is undefined in the reference
        # (it reads past its arrays): stay below it, and put 40 samples in the
        # face cells n-2 of each axis, where the face rule of the derivatives applies
        last = np.floor(center - 10.5) + 20.0  # first coordinate of cell n-1 (n = 21)
        pts = np.minimum(pts, last - 0.01)
        for d in range(3):
            pts[40 * d:40 * (d + 1), d] = last[d] - 1.0 + rng.uniform(0.0, 0.99, 40)
        for it in range(3):
            out[f"interp_{vs}_{it}_pts"] = pts
            out[f"interp_{vs}_{it}_val"] = R.interpolate(p, vcor, center, pts, it)
            out[f"interp_{vs}_{it}_center"] = center
    # objectives
    r = rng.uniform(0, 255, 500)
    t = r + rng.normal(0, 10, 500)
    out["obj_ref"] = r
    out["obj_tar"] = t
    for f in range(5):
        o, res = R.objective(f, r, t, True)
        out[f"obj_{f}_val"] = np.array([o])
        out[f"obj_{f}_res"] = res
    # searches
    pts = synth.grid_points((3, 3, 3), 5.0, (20.0, 20.0, 20.0))
    O = Oracle()
    order, neigh = R.order_neighbours(pts)
    for k, (vs, kw) in enumerate(SEARCH_CASES):
        vref, vcor = vols[vs]
        bpv = 1 if vref.dtype == np.uint8 else 2
        p = make_params(SHAPE, bytes_per_voxel=bpv, **kw)
        res = R.process(p, vref, cor=vcor, points=pts, order=order, neigh=neigh)
        out[f"search_{k}_status"] = res["status"]
        out[f"search_{k}_objmin"] = res["objmin"]
        out[f"search_{k}_params"] = res["params"]
    out["search_points"] = pts
    out["search_order"] = order
    out["search_neigh"] = neigh
    for vs, (vref, vcor) in vols.items():
        out[f"vol_{vs}_ref"] = vref
        out[f"vol_{vs}_cor"] = vcor
    np.savez_compressed(os.path.join(HERE, "reference_hotpath.npz"), **out)
    with open(os.path.join(HERE, "search_cases.json"), "w") as f:
        json.dump([dict(volumes=vs, **kw) for vs, kw in SEARCH_CASES], f, indent=1)
    with tempfile.TemporaryDirectory() as tmp:
        st = strain_golden(tmp)
    np.savez_compressed(os.path.join(HERE, "reference_strain.npz"),
                        **{f"{c}_{k}": np.asarray(v) for c, d in st.items() for k, v in d.items()})
    with open(os.path.join(HERE, "datacloud_knn.json"), "w") as f:
        json.dump(datacloud_golden(), f, indent=1)
    with tempfile.TemporaryDirectory() as tmp:
        runs = dvc_runs_golden(tmp, vols)
    with open(os.path.join(HERE, "dvc_runs.json"), "w") as f:
        json.dump(runs, f, indent=1)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
