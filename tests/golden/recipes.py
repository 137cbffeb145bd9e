"""Recipes of the larger golden cases: seeded synthetic volume pairs, point
grids and search settings, rendered on demand (numpy) instead of stored.

make_golden.py runs the reference's own code (oracle/_ref) on them and
records its outputs together with a SHA-256 digest of each rendered volume
pair; the tests render the same volumes, check the digest, and compare the
GPU engine with the recorded outputs.

  RANGE_CASES   searches in which the reference reports Range_Fail (-1),
                one family per route by which its search leaves the active
                interpolation box (BoundBox::contains in tri_cub_Lek,
                Core/Interpolate.cpp:474-481): Gauss-Newton translating the
                subvolume out (no grid; grid + Gauss-Newton), and 12-dof
                Gauss-Newton whose rotation or strain grows the warped cloud's
                bounding box (FloatingCloud::resize_bbox, Core/FloatingCloud.cpp:
                206-233) out of the box. The failing clouds leave through the
                box's low faces: near its high faces the reference reads past
                its coefficient array (the last cell plane, an undefined
                result), so those cases would pin nothing.
  LARGE_CASES   full-size subvolumes on a 128^3 uint16 crop: sphere 41 /
                4000 samples / 12 dof (the precision + scale workload's) and
                cube 41 / 3375 samples / 12 dof (the full pipeline's).
  CONFIG1       the plain-method workload end to end through the `dvc`
                program: 256^3 uint8, 1000 points, cube 31 / 2197 samples.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from digitalvolumecorrelation_gb300 import synth  # noqa: E402

U8 = dict(amp=(40.0, 200.0), dtype="uint8", noise=2.0)
U16 = dict(amp=(2000.0, 60000.0), dtype="uint16", noise=150.0)
GRID48 = dict(n=(4, 4, 3), spacing=10.0, centre=(32.0, 32.0, 32.0))
GRID27 = dict(n=(3, 3, 3), spacing=4.0, centre=(32.0, 32.0, 32.0))


def _case(name, vol, deform, grid, **params):
    return dict(name=name, volume=vol, deform=deform, grid=grid, params=params)


VOL64 = dict(shape=(64, 64, 64), n_blobs=900, seeds=(71, 72, 73))
RANGE_CASES = [
    _case("gn_translation_6dof", dict(VOL64, **U8),
          dict(kind="piecewise", t1=(0.3, -0.2, 0.1), t2=(-3.4, -0.4, 0.3), split=32.0), GRID48,
          subvol_geom="cube", subvol_size=11, subvol_npts=343, obj_function="znssd",
          interp_type="tricubic", num_srch_dof=6, disp_max=1, basin_radius=0.0),
    _case("gn_translation_3dof", dict(VOL64, **U8),
          dict(kind="piecewise", t1=(0.3, -0.2, 0.1), t2=(-4.4, -0.4, 0.3), split=32.0), GRID48,
          subvol_geom="cube", subvol_size=11, subvol_npts=343, obj_function="znssd",
          interp_type="tricubic", num_srch_dof=3, disp_max=2, basin_radius=0.0),
    _case("gn_translation_u16_sphere", dict(VOL64, **U16),
          dict(kind="piecewise", t1=(0.3, -0.2, 0.1), t2=(-4.4, -0.4, 0.3), split=32.0), GRID48,
          subvol_geom="sphere", subvol_size=11, subvol_npts=400, obj_function="zssd",
          interp_type="tricubic", num_srch_dof=6, disp_max=2, basin_radius=0.0),
    _case("grid_then_gn", dict(VOL64, **U8),
          dict(kind="piecewise", t1=(0.3, -0.2, 0.1), t2=(4.2, 0.4, -0.3), split=32.0), GRID48,
          subvol_geom="cube", subvol_size=11, subvol_npts=343, obj_function="znssd",
          interp_type="tricubic", num_srch_dof=3, disp_max=2, basin_radius=1.0),
    _case("rotation_12dof", dict(VOL64, **U8),
          dict(kind="affine", t=(-1.6, -1.6, 0.0), rot_z_deg=14.0, c=(32.0, 32.0, 32.0)), GRID27,
          subvol_geom="cube", subvol_size=21, subvol_npts=1000, obj_function="znssd",
          interp_type="tricubic", num_srch_dof=12, disp_max=1, basin_radius=0.0),
    _case("strain_12dof", dict(VOL64, **U8),
          dict(kind="affine", t=(0.0, 0.0, -1.2), E=((0, 0, 0), (0, 0, 0), (0, 0, 0.2)),
               c=(32.0, 32.0, 32.0)), GRID27,
          subvol_geom="sphere", subvol_size=21, subvol_npts=1500, obj_function="znssd",
          interp_type="tricubic", num_srch_dof=12, disp_max=1, basin_radius=0.0),
]

GRID128 = dict(n=(3, 3, 3), spacing=16.0, centre=(64.0, 64.0, 64.0))
LARGE_CASES = [
    _case("sphere41_4000_12dof", dict(shape=(128, 128, 128), n_blobs=2097, seeds=(81, 82, 83), **U16),
          dict(kind="sinusoid", A=3.0, L=160.0), GRID128,
          subvol_geom="sphere", subvol_size=41, subvol_npts=4000, obj_function="znssd",
          interp_type="tricubic", num_srch_dof=12, disp_max=6, basin_radius=3.0),
    _case("cube41_3375_12dof", dict(shape=(128, 128, 128), n_blobs=2097, seeds=(91, 92, 93), **U16),
          dict(kind="bendjump", kappa=1e-3, xc=64.0, h=256.0, J=2.0, z0=64.0, w=5.0), GRID128,
          subvol_geom="cube", subvol_size=41, subvol_npts=3000, obj_function="znssd",
          interp_type="tricubic", num_srch_dof=12, disp_max=6, basin_radius=3.0),
]

# a `dvc` program run over a Range_Fail case: .disp rows of failed points
RANGE_DVC_RUN = dict(case="gn_translation_6dof", header=0, endian="little",
                     roi_extra="", labels_seed=4)


def deform(spec):
    k = spec["kind"]
    if k == "piecewise":
        return synth.Piecewise(t1=spec["t1"], t2=spec["t2"], split=spec["split"])
    if k == "affine":
        E = synth.rotation_z(spec["rot_z_deg"]) if "rot_z_deg" in spec else spec["E"]
        return synth.Affine(t=spec["t"], E=E, c=spec["c"])
    if k == "sinusoid":
        return synth.Sinusoid(A=spec["A"], L=spec["L"])
    if k == "bendjump":
        return synth.BendJump(kappa=spec["kappa"], xc=spec["xc"], h=spec["h"], J=spec["J"],
                              z0=spec["z0"], w=spec["w"])
    raise ValueError(k)


def render(case):
    """(reference, correlate) volumes [z, y, x] of a case."""
    v = case["volume"]
    dt = np.uint8 if v["dtype"] == "uint8" else np.uint16
    b = synth.blobs(tuple(v["shape"]), v["n_blobs"], amp=tuple(v["amp"]), seed=v["seeds"][0])
    ref = synth.render(tuple(v["shape"]), b, noise_sigma=v["noise"], noise_seed=v["seeds"][1], dtype=dt)
    cor = synth.render(tuple(v["shape"]), b, deform=deform(case["deform"]), noise_sigma=v["noise"],
                       noise_seed=v["seeds"][2], dtype=dt)
    return ref, cor


def points(case):
    g = case["grid"]
    return synth.grid_points(tuple(g["n"]), g["spacing"], tuple(g["centre"]))


def digest(ref, cor):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(ref).tobytes())
    h.update(np.ascontiguousarray(cor).tobytes())
    return h.hexdigest()


def params(case):
    from digitalvolumecorrelation_gb300.abi import make_params
    v = case["volume"]
    return make_params(tuple(v["shape"]), bytes_per_voxel=1 if v["dtype"] == "uint8" else 2,
                       **case["params"])


def by_name(name):
    for c in RANGE_CASES + LARGE_CASES:
        if c["name"] == name:
            return c
    raise KeyError(name)


def config1_volumes():
    """The plain-method workload's pair (256^3 uint8), rendered with numpy."""
    from digitalvolumecorrelation_gb300 import workloads
    W = workloads.config1()
    ref = synth.render(W.shape, W.blobs, noise_sigma=W.noise_sigma, noise_seed=W.ref_seed)
    cor = synth.render(W.shape, W.blobs, deform=W.deform, noise_sigma=W.noise_sigma,
                       noise_seed=W.cor_seed)
    return W, ref, cor
