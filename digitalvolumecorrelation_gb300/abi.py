"""ctypes mirror of include/dvc_gpu.h (structs, enums, status codes)."""
from __future__ import annotations

import ctypes as C

POINT_GOOD, RANGE_FAIL, CONVG_FAIL, NOT_SEARCH = 0, -1, -2, -3
OK, E_ARG, E_CUDA, E_NOMEM, E_TIMEOUT, E_RANGE = 0, -10, -11, -12, -13, -14

OBJ = {"sad": 0, "ssd": 1, "zssd": 2, "nssd": 3, "znssd": 4}
INTERP = {"nearest": 0, "trilinear": 1, "tricubic": 2}
GEOM = {"cube": 0, "sphere": 1}
SEED_NEIGHBOURS, SEED_GIVEN, SEED_RIGID, SEED_PARAMS = 0, 1, 2, 3
COARSE = {"grid": 0, "random": 1}
REFINE = {"gauss_newton": 0, "nelder_mead": 1}


class DvcParams(C.Structure):
    _fields_ = [
        ("vol_wide", C.c_int), ("vol_high", C.c_int), ("vol_tall", C.c_int),
        ("bytes_per_voxel", C.c_int),
        ("subvol_geom", C.c_int), ("subvol_size", C.c_int), ("subvol_npts", C.c_int),
        ("subvol_aspect", C.c_double * 3),
        ("disp_max", C.c_int), ("num_srch_dof", C.c_int),
        ("obj_function", C.c_int), ("interp_type", C.c_int),
        ("basin_radius", C.c_double), ("rigid_trans", C.c_double * 3),
        ("sphere_seed", C.c_uint),
        ("subvol_thresh", C.c_int), ("gray_thresh_min", C.c_double), ("gray_thresh_max", C.c_double),
        ("min_vol_fract", C.c_double),
        ("coarse_method", C.c_int), ("refine_method", C.c_int), ("coarse_seed", C.c_uint),
    ]


class DvcStats(C.Structure):
    _fields_ = [
        ("n_processed", C.c_int), ("n_good", C.c_int), ("n_range_fail", C.c_int),
        ("n_convg_fail", C.c_int), ("n_evaluations", C.c_longlong),
        ("n_gn_iterations", C.c_longlong), ("kernel_ms", C.c_double), ("total_ms", C.c_double),
    ]


def make_params(shape_xyz, bytes_per_voxel=1, subvol_geom="cube", subvol_size=31,
                subvol_npts=2000, subvol_aspect=(1.0, 1.0, 1.0), disp_max=12, num_srch_dof=6,
                obj_function="znssd", interp_type="tricubic", basin_radius=0.0,
                rigid_trans=(0.0, 0.0, 0.0), sphere_seed=1, subvol_thresh=False, gray_thresh_min=25.0,
                gray_thresh_max=125.0, min_vol_fract=0.2, coarse_method="grid",
                refine_method="gauss_newton", coarse_seed=1) -> DvcParams:
    p = DvcParams()
    p.vol_wide, p.vol_high, p.vol_tall = (int(v) for v in shape_xyz)
    p.bytes_per_voxel = int(bytes_per_voxel)
    p.subvol_geom = GEOM[subvol_geom] if isinstance(subvol_geom, str) else int(subvol_geom)
    p.subvol_size = int(subvol_size)
    p.subvol_npts = int(subvol_npts)
    p.subvol_aspect[:] = [float(v) for v in subvol_aspect]
    p.disp_max = int(disp_max)
    p.num_srch_dof = int(num_srch_dof)
    p.obj_function = OBJ[obj_function] if isinstance(obj_function, str) else int(obj_function)
    p.interp_type = INTERP[interp_type] if isinstance(interp_type, str) else int(interp_type)
    p.basin_radius = float(basin_radius)
    p.rigid_trans[:] = [float(v) for v in rigid_trans]
    p.sphere_seed = int(sphere_seed)
    p.subvol_thresh = int(bool(subvol_thresh))
    p.gray_thresh_min = float(gray_thresh_min)
    p.gray_thresh_max = float(gray_thresh_max)
    p.min_vol_fract = float(min_vol_fract)
    p.coarse_method = COARSE[coarse_method] if isinstance(coarse_method, str) else int(coarse_method)
    p.refine_method = REFINE[refine_method] if isinstance(refine_method, str) else int(refine_method)
    p.coarse_seed = int(coarse_seed)
    return p
