"""Loaders for the golden fixtures recorded from the reference (tests/golden)."""
import json
import os

import numpy as np

from digitalvolumecorrelation_gb300.abi import make_params

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SHAPE = (40, 40, 40)


def hotpath():
    return np.load(os.path.join(GOLDEN, "reference_hotpath.npz"))


def search_cases():
    with open(os.path.join(GOLDEN, "search_cases.json")) as f:
        return json.load(f)


def case_params(case):
    kw = {k: v for k, v in case.items() if k != "volumes"}
    d = hotpath()
    bpv = 1 if d[f"vol_{case['volumes']}_ref"].dtype == np.uint8 else 2
    return make_params(SHAPE, bytes_per_voxel=bpv, **kw)


def interp_params(vs):
    d = hotpath()
    bpv = 1 if d[f"vol_{vs}_ref"].dtype == np.uint8 else 2
    return make_params(SHAPE, bytes_per_voxel=bpv, subvol_size=11, subvol_npts=300, disp_max=3)


def strain_cases():
    d = np.load(os.path.join(GOLDEN, "reference_strain.npz"))
    names = sorted({k.split("_")[0] if not k.startswith("vol_t") else "vol_t" for k in d.files})
    out = {}
    for name in ("vol", "vol_t", "planar"):
        pre = name + "_"
        out[name] = {k[len(pre):]: d[k] for k in d.files
                     if k.startswith(pre) and not (name == "vol" and k.startswith("vol_t_"))}
    return out


def strain_flags(args):
    args = [str(a) for a in args]
    ndp = 25
    objt = 1.0
    refill = "-r" in args
    if "-sw" in args:
        ndp = min(max(int(args[args.index("-sw") + 1]), 10), 75)
    if "-t" in args:
        objt = min(max(float(args[args.index("-t") + 1]), 0.0001), 1.0)
    return ndp, objt, refill


def planar_flag(pts):
    flag = 0
    if abs(pts[:, 0].max() - pts[:, 0].min()) < 0.001:
        flag |= 1
    if abs(pts[:, 1].max() - pts[:, 1].min()) < 0.001:
        flag |= 2
    if abs(pts[:, 2].max() - pts[:, 2].min()) < 0.001:
        flag |= 4
    return flag
