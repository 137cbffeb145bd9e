"""Python mirror of the reference's hot-path interface over libdvcgpu.so.

The reference exposes its hot path as C++ classes used by the `dvc` and
`strain` programs: Search (process_point over the ROI points,
Core/Search.cpp:95-192), Interpolate (nearest / tri_lin / tri_cub_Lek,
Core/Interpolate.cpp:404-567), the objective functions
(Core/ObjectiveFunctions.cpp) and the strain fit (Core/strain.cpp:402-591).
This module binds the C ABI of include/dvc_gpu.h with ctypes and keeps the
reference's names and argument meaning. There is no CPU path: every call runs
on the GPU, and loading fails loudly when the CUDA library is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .abi import (DvcParams, DvcStats, E_ARG, E_RANGE, OK, SEED_GIVEN, SEED_NEIGHBOURS, SEED_PARAMS,
                  SEED_RIGID, make_params)

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libdvcgpu.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lib = None


class DvcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"dvc_gpu error {code}: {msg}")
        self.code = code


def load(path: str | None = None):
    """Load libdvcgpu.so (built by digitalvolumecorrelation_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"CUDA library {p} is missing: run `python -m "
                           "digitalvolumecorrelation_gb300.build` (no CPU fallback exists)")
    L = C.CDLL(p)
    L.dvc_gpu_version.restype = C.c_char_p
    L.dvc_gpu_last_error.restype = C.c_char_p
    L.dvc_gpu_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(DvcParams), C.c_void_p,
                                 C.c_void_p, C.c_int]
    L.dvc_gpu_create_device.argtypes = [C.POINTER(C.c_void_p), C.POINTER(DvcParams), C.c_void_p,
                                        C.c_void_p]
    L.dvc_gpu_destroy.argtypes = [C.c_void_p]
    L.dvc_gpu_destroy.restype = None
    L.dvc_gpu_process.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, _ip, C.c_int, _ip, C.c_int,
                                  _dp, _ip, _dp, _dp, _ip, C.POINTER(DvcStats)]
    L.dvc_gpu_process_device.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                         C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.dvc_gpu_last_counters.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
    L.dvc_gpu_last_phase_cycles.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
    L.dvc_gpu_last_status.argtypes = [C.c_void_p]
    L.dvc_gpu_set_wait_limit.argtypes = [C.c_void_p, C.c_longlong]
    L.dvc_gpu_interpolate.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, _dp, C.c_int, _dp]
    L.dvc_gpu_objective.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp]
    L.dvc_gpu_strain.argtypes = [C.c_int, _dp, _ip, _dp, _dp, C.c_int, _ip, C.c_int, C.c_double,
                                 C.c_int, C.c_int, _dp, _ip, _dp, _dp, _dp, _dp]
    L.dvc_cnn_create.argtypes = [C.POINTER(C.c_void_p), C.c_uint]
    L.dvc_cnn_destroy.argtypes = [C.c_void_p]
    L.dvc_cnn_destroy.restype = None
    L.dvc_cnn_get_weights.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int]
    L.dvc_cnn_set_weights.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int]
    L.dvc_cnn_patches.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.dvc_cnn_forward.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.dvc_cnn_gradients.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(C.c_float),
                                    C.POINTER(C.c_float)]
    L.dvc_cnn_train_step.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_float,
                                     C.POINTER(C.c_float)]
    L.dvc_gpu_process_learned.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                          C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.POINTER(C.c_int), C.c_void_p]
    L.dvc_gpu_order_neighbours.argtypes = [C.c_int, _dp, _dp, C.c_int, _ip, _ip]
    L.dvc_gpu_set_cluster.argtypes = [C.c_void_p, C.c_int]
    L.dvc_gpu_last_launch.argtypes = [C.c_void_p, _ip]
    L.dvc_gpu_last_windows.argtypes = [C.c_void_p, _ip]
    L.dvc_gpu_read_mhd.argtypes = [C.c_char_p, C.POINTER(DvcVolumeInfo)]
    L.dvc_gpu_load_raw.argtypes = [C.c_void_p, C.c_char_p, C.c_longlong, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_int, C.c_void_p]
    L.dvc_gpu_create_from_files.argtypes = [C.POINTER(C.c_void_p), C.POINTER(DvcParams), C.c_char_p,
                                            C.c_char_p, C.c_longlong, C.c_int]
    L.dvc_gpu_plan_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int, C.c_int]
    L.dvc_gpu_plan_destroy.argtypes = [C.c_void_p]
    L.dvc_gpu_plan_destroy.restype = None
    L.dvc_gpu_plan_info.argtypes = [C.c_void_p, _ip, _ip, _ip, C.POINTER(C.c_longlong)]
    L.dvc_gpu_plan_set_shape.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.dvc_gpu_plan_process_device.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                              C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.dvc_gpu_plan_process.argtypes = [C.c_void_p, _ip, C.c_int, _dp, C.c_int, _ip, C.c_int, _ip, C.c_int,
                                       _dp, _ip, _dp, _dp, _ip, C.POINTER(DvcStats)]
    L.dvc_gpu_plan_autotune.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                        C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_int, _dp]
    L.dvc_gpu_synth_volume.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.POINTER(C.c_float), C.c_int, _dp, C.c_float, C.c_float,
                                       C.c_ulonglong, C.c_float, C.c_void_p]
    _lib = L
    return L


def _check(rc):
    if rc != OK:
        raise DvcError(rc, _lib.dvc_gpu_last_error().decode())


def _p(a, t):
    return a.ctypes.data_as(t)


class DvcVolumeInfo(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("bytes_per_voxel", C.c_int),
                ("big_endian", C.c_int), ("header_bytes", C.c_longlong), ("data_file", C.c_char * 1024)]


def read_mhd(path):
    """MetaImage header (dvc_gpu_read_mhd): dict(nx, ny, nz, bytes_per_voxel,
    big_endian, header_bytes, data_file)."""
    load()
    info = DvcVolumeInfo()
    _check(_lib.dvc_gpu_read_mhd(os.fsencode(path), C.byref(info)))
    return dict(nx=info.nx, ny=info.ny, nz=info.nz, bytes_per_voxel=info.bytes_per_voxel,
                big_endian=info.big_endian, header_bytes=info.header_bytes,
                data_file=info.data_file.decode())


def load_raw(vol_dev, path, shape_xyz, bytes_per_voxel, header_bytes=0, big_endian=False, stream=0):
    """Stream a raw volume file into a device buffer (dvc_gpu_load_raw)."""
    load()
    nx, ny, nz = shape_xyz
    _check(_lib.dvc_gpu_load_raw(C.c_void_p(_dev_ptr(vol_dev)), os.fsencode(path), int(header_bytes), nx, ny,
                                 nz, int(bytes_per_voxel), int(big_endian), C.c_void_p(stream)))


class Engine:
    """Both volumes resident on the GPU; Search::Search + Interpolate."""

    def __init__(self, params: DvcParams, ref=None, cor=None, big_endian=False, ref_dev=None,
                 cor_dev=None, ref_path=None, cor_path=None, header_bytes=0):
        L = load()
        self.params = params
        self._h = C.c_void_p()
        self._keep = []
        if ref_path is not None:
            _check(L.dvc_gpu_create_from_files(C.byref(self._h), C.byref(params), os.fsencode(ref_path),
                                               os.fsencode(cor_path), int(header_bytes), int(big_endian)))
        elif ref_dev is not None:
            # device buffers (e.g. torch CUDA tensors): pass their addresses
            self._keep = [ref_dev, cor_dev]
            _check(L.dvc_gpu_create_device(C.byref(self._h), C.byref(params),
                                           C.c_void_p(_dev_ptr(ref_dev)), C.c_void_p(_dev_ptr(cor_dev))))
        else:
            ref = np.ascontiguousarray(ref)
            cor = np.ascontiguousarray(cor)
            _check(L.dvc_gpu_create(C.byref(self._h), C.byref(params),
                                    ref.ctypes.data_as(C.c_void_p), cor.ctypes.data_as(C.c_void_p),
                                    int(big_endian)))

    def close(self):
        if self._h:
            _lib.dvc_gpu_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_cluster(self, cluster):
        """CTAs per point for this engine's searches (1, 2, 4, 8; 0: chosen per call)."""
        _check(_lib.dvc_gpu_set_cluster(self._h, int(cluster)))

    def process(self, points, order=None, neigh=None, n_process=None, seed_mode=SEED_NEIGHBOURS,
                seeds=None):
        """Search::process_point over `order` (Core/dvc.cpp:233-303)."""
        return _host_search(lambda *args: _lib.dvc_gpu_process(self._h, *args), points, order, neigh,
                            n_process, seed_mode, seeds)

    def process_device(self, n_points, points_dev, order_dev, n_process, neigh_dev, n_neigh,
                       seed_mode, seeds_dev, status_dev, objmin_dev, params_dev, gn_iters_dev=None,
                       stream=0):
        """Device-resident variant (torch CUDA tensors or raw pointers)."""
        ptr = lambda t: C.c_void_p(_dev_ptr(t)) if t is not None else None
        _check(_lib.dvc_gpu_process_device(self._h, int(n_points), ptr(points_dev), int(n_process),
                                           ptr(order_dev), int(n_neigh), ptr(neigh_dev),
                                           int(seed_mode), ptr(seeds_dev), ptr(status_dev),
                                           ptr(objmin_dev), ptr(params_dev), ptr(gn_iters_dev),
                                           C.c_void_p(stream)))

    def process_learned(self, net, n_points, points_dev, order_dev, n_process, obj_threshold,
                        status_dev, objmin_dev, params_dev, gn_iters_dev=None, stream=0):
        """The learned search (dvc_gpu_process_learned); returns the number of
        points searched again by the plain method."""
        ptr = lambda t: C.c_void_p(_dev_ptr(t)) if t is not None else None
        nfb = C.c_int(0)
        _check(_lib.dvc_gpu_process_learned(self._h, net._h, int(n_points), ptr(points_dev),
                                            int(n_process), ptr(order_dev), float(obj_threshold),
                                            ptr(status_dev), ptr(objmin_dev), ptr(params_dev),
                                            ptr(gn_iters_dev), C.byref(nfb), C.c_void_p(stream)))
        return nfb.value

    def last_launch(self):
        """dict(cluster, ctas, staging (0 none, 1 every translation, 2 per z
        slab), smem_bytes) of the most recent search launch."""
        out = (C.c_int * 4)()
        _check(_lib.dvc_gpu_last_launch(self._h, out))
        return dict(cluster=out[0], ctas=out[1], staging=out[2], smem_bytes=out[3])

    def last_windows(self):
        """(w1, w2, width) of the most recent search with the reference's
        seeding: ranks [0, w1) and [w2, n) searched at `width` CTAs per point,
        the ranks between at last_launch()["cluster"]; w1 = w2 = n: one launch."""
        out = (C.c_int * 3)()
        _check(_lib.dvc_gpu_last_windows(self._h, out))
        return tuple(out)

    def last_counters(self):
        """(evaluations, Gauss-Newton iterations, undefined-cell evaluations)
        of the most recent search on this engine."""
        out = (C.c_longlong * 3)()
        _check(_lib.dvc_gpu_last_counters(self._h, out))
        return tuple(int(v) for v in out)

    def last_status(self):
        """Device-side outcome of the most recent search launch
        (dvc_gpu_last_status): OK, or the DVC_E_* code it recorded."""
        return int(_lib.dvc_gpu_last_status(self._h))

    def set_wait_limit(self, polls):
        """Polls before a dependency wait of the search gives up (< 0: default)."""
        _check(_lib.dvc_gpu_set_wait_limit(self._h, int(polls)))

    def last_phase_cycles(self):
        """SM cycles of the most recent search per phase, summed over CTAs:
        (seed, setup, grid, gn_entry_exit, final, gn_warp, gn_range_stage,
        gn_eval, gn_reduce, gn_solve, gn_gtg)."""
        out = (C.c_longlong * 11)()
        _check(_lib.dvc_gpu_last_phase_cycles(self._h, out))
        return tuple(int(v) for v in out)

    def interpolate(self, volume, center, pts, interp_type=2):
        """Interpolate::center_on + nearest/tri_lin/tri_cub_Lek; None on Intrp_Fail."""
        pts = np.ascontiguousarray(pts, np.float64)
        out = np.zeros(len(pts))
        c = np.ascontiguousarray(center, np.float64)
        rc = _lib.dvc_gpu_interpolate(self._h, int(volume), _p(c, _dp), len(pts), _p(pts, _dp),
                                      int(interp_type), _p(out, _dp))
        if rc == E_RANGE:
            return None
        _check(rc)
        return out


def _host_search(call, points, order, neigh, n_process, seed_mode, seeds):
    """Host arrays in, the C search call, result arrays and stats out."""
    pts = np.ascontiguousarray(points, np.float64)
    n = len(pts)
    order = np.arange(n, dtype=np.int32) if order is None else np.ascontiguousarray(order, np.int32)
    n_process = len(order) if n_process is None else int(n_process)
    nn = 0
    neigh_p = None
    if neigh is not None and seed_mode == SEED_NEIGHBOURS:
        neigh = np.ascontiguousarray(neigh, np.int32)
        nn = neigh.shape[1]
        neigh_p = _p(neigh, _ip)
    seeds_p = None
    if seed_mode in (SEED_GIVEN, SEED_PARAMS):
        seeds = np.ascontiguousarray(seeds, np.float64)
        seeds_p = _p(seeds, _dp)
    status = np.zeros(n, np.int32)
    objmin = np.zeros(n)
    par = np.zeros((n, 12))
    its = np.zeros(n, np.int32)
    st = DvcStats()
    _check(call(n, _p(pts, _dp), n_process, _p(order, _ip), nn, neigh_p, int(seed_mode), seeds_p,
                _p(status, _ip), _p(objmin, _dp), _p(par, _dp), _p(its, _ip), C.byref(st)))
    return dict(status=status, objmin=objmin, params=par, gn_iters=its,
                stats={f: getattr(st, f) for f, _ in DvcStats._fields_})


class Plan:
    """Several search configurations (engines on the same volumes) searched in
    one launch, each point by its own configuration (dvc_gpu_plan_*)."""

    def __init__(self, engines, cluster=0):
        L = load()
        self.engines = list(engines)  # the plan uses their sample tables
        arr = (C.c_void_p * len(self.engines))(*[e._h.value for e in self.engines])
        self._h = C.c_void_p()
        _check(L.dvc_gpu_plan_create(C.byref(self._h), arr, len(self.engines), int(cluster)))

    def close(self):
        if self._h:
            _lib.dvc_gpu_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        """dict(cluster, staging, n_staged, smem_bytes) of the launch shape."""
        c, s, n = C.c_int(), C.c_int(), C.c_int()
        m = C.c_longlong()
        _check(_lib.dvc_gpu_plan_info(self._h, C.byref(c), C.byref(s), C.byref(n), C.byref(m)))
        return dict(cluster=c.value, staging=s.value, n_staged=n.value, smem_bytes=m.value)

    def set_shape(self, cluster, staging=1):
        _check(_lib.dvc_gpu_plan_set_shape(self._h, int(cluster), int(staging)))

    def process(self, point_cfg, points, order=None, neigh=None, n_process=None,
                seed_mode=SEED_NEIGHBOURS, seeds=None):
        cfg = np.ascontiguousarray(point_cfg, np.int32)
        return _host_search(lambda *args: _lib.dvc_gpu_plan_process(self._h, _p(cfg, _ip), *args), points,
                            order, neigh, n_process, seed_mode, seeds)

    def process_device(self, point_cfg_dev, n_points, points_dev, order_dev, n_process, neigh_dev, n_neigh,
                       seed_mode, seeds_dev, status_dev, objmin_dev, params_dev, gn_iters_dev=None,
                       stream=0):
        ptr = lambda t: C.c_void_p(_dev_ptr(t)) if t is not None else None
        _check(_lib.dvc_gpu_plan_process_device(self._h, ptr(point_cfg_dev), int(n_points), ptr(points_dev),
                                                int(n_process), ptr(order_dev), int(n_neigh), ptr(neigh_dev),
                                                int(seed_mode), ptr(seeds_dev), ptr(status_dev),
                                                ptr(objmin_dev), ptr(params_dev), ptr(gn_iters_dev),
                                                C.c_void_p(stream)))

    def autotune(self, point_cfg_dev, n_points, points_dev, order_dev, n_process, neigh_dev, n_neigh,
                 seed_mode, seeds_dev, status_dev, objmin_dev, params_dev, reps=2):
        """Time every launch shape on these points and keep the fastest;
        returns {(cluster, staging): mean ms} of the shapes that fit."""
        ptr = lambda t: C.c_void_p(_dev_ptr(t)) if t is not None else None
        ms = np.zeros(8)
        _check(_lib.dvc_gpu_plan_autotune(self._h, ptr(point_cfg_dev), int(n_points), ptr(points_dev),
                                          int(n_process), ptr(order_dev), int(n_neigh), ptr(neigh_dev),
                                          int(seed_mode), ptr(seeds_dev), ptr(status_dev), ptr(objmin_dev),
                                          ptr(params_dev), int(reps), _p(ms, _dp)))
        return {(1 << (j // 2), j % 2): float(ms[j]) for j in range(8) if ms[j] >= 0}


class Cnn:
    """The learned initial-guess network (dvc_cnn_* of dvc_gpu.h)."""

    def __init__(self, seed=1):
        L = load()
        self._h = C.c_void_p()
        _check(L.dvc_cnn_create(C.byref(self._h), int(seed)))
        self.n_params = L.dvc_cnn_param_count()

    def close(self):
        if self._h:
            _lib.dvc_cnn_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_weights(self):
        w = np.zeros(self.n_params, np.float32)
        _check(_lib.dvc_cnn_get_weights(self._h, w.ctypes.data_as(C.POINTER(C.c_float)), self.n_params))
        return w

    def set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        _check(_lib.dvc_cnn_set_weights(self._h, w.ctypes.data_as(C.POINTER(C.c_float)), len(w)))

    @staticmethod
    def patches(engine, n, points_dev, patches_dev, idx_dev=None, stream=0):
        """[n][2][32][32][32] patches of an engine's volume pair (device)."""
        load()
        _check(_lib.dvc_cnn_patches(engine._h, int(n), C.c_void_p(_dev_ptr(points_dev)),
                                    C.c_void_p(_dev_ptr(idx_dev)) if idx_dev is not None else None,
                                    C.c_void_p(_dev_ptr(patches_dev)), C.c_void_p(stream)))

    def forward(self, batch, patches_dev, out_dev, stream=0):
        _check(_lib.dvc_cnn_forward(self._h, int(batch), C.c_void_p(_dev_ptr(patches_dev)),
                                    C.c_void_p(_dev_ptr(out_dev)), C.c_void_p(stream)))

    def gradients(self, batch, patches_dev, targets_dev):
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_float(0.0)
        _check(_lib.dvc_cnn_gradients(self._h, int(batch), C.c_void_p(_dev_ptr(patches_dev)),
                                      C.c_void_p(_dev_ptr(targets_dev)),
                                      g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)))
        return g, loss.value

    def train_step(self, batch, patches_dev, targets_dev, lr):
        loss = C.c_float(0.0)
        _check(_lib.dvc_cnn_train_step(self._h, int(batch), C.c_void_p(_dev_ptr(patches_dev)),
                                       C.c_void_p(_dev_ptr(targets_dev)), float(lr), C.byref(loss)))
        return loss.value


def _dev_ptr(t):
    if isinstance(t, int):
        return t
    return int(t.data_ptr())


def objective(fcn, ref, tar, residual=False):
    """obj_SAD .. obj_ZNSSD on the GPU (FP64)."""
    load()
    ref = np.ascontiguousarray(ref, np.float64)
    tar = np.ascontiguousarray(tar, np.float64)
    o = C.c_double()
    res = np.zeros(len(ref)) if residual else None
    _check(_lib.dvc_gpu_objective(int(fcn), len(ref), _p(ref, _dp), _p(tar, _dp), C.byref(o),
                                  _p(res, _dp) if residual else None))
    return (o.value, res) if residual else o.value


def strain(pts, status, objmin, disp, neigh, ndp=25, objt=1.0, refill=False, planar=0):
    """Strain-window fit of the `strain` program (Core/strain.cpp:402-591)."""
    load()
    n = len(pts)
    pts = np.ascontiguousarray(pts, np.float64)
    status = np.ascontiguousarray(status, np.int32)
    objmin = np.ascontiguousarray(objmin, np.float64)
    disp = np.ascontiguousarray(disp, np.float64)
    neigh = np.ascontiguousarray(neigh, np.int32)
    out = dict(u_fit=np.zeros((n, 3)), pts_in_sw=np.zeros(n, np.int32), sw_radius=np.zeros(n),
               e_strain=np.zeros((n, 9)), l_strain=np.zeros((n, 9)), dgrad=np.zeros((n, 9)))
    _check(_lib.dvc_gpu_strain(n, _p(pts, _dp), _p(status, _ip), _p(objmin, _dp), _p(disp, _dp),
                               neigh.shape[1], _p(neigh, _ip), int(ndp), float(objt), int(refill),
                               int(planar), _p(out["u_fit"], _dp), _p(out["pts_in_sw"], _ip),
                               _p(out["sw_radius"], _dp), _p(out["e_strain"], _dp),
                               _p(out["l_strain"], _dp), _p(out["dgrad"], _dp)))
    return out


def order_neighbours(points, start=None, k=75):
    """Processing order by distance from `start` (default the first point) and
    the k nearest points of every point, on the GPU (ties by index)."""
    load()
    pts = np.ascontiguousarray(points, np.float64)
    n = len(pts)
    s = np.ascontiguousarray(pts[0] if start is None else start, np.float64)
    kk = min(k, n)
    order = np.zeros(n, np.int32)
    neigh = np.zeros((n, kk), np.int32)
    _check(_lib.dvc_gpu_order_neighbours(n, _p(pts, _dp), _p(s, _dp), int(k), _p(order, _ip),
                                         _p(neigh, _ip)))
    return order, neigh


def synth_volume_device(vol_dev, shape_xyz, bytes_per_voxel, blobs, deform=None,
                        background=0.0, noise_sigma=2.0, noise_seed=1, vmax=None, stream=0):
    """Render a speckle volume into a device buffer (see dvc_gpu_synth_volume)."""
    load()
    b = np.ascontiguousarray(blobs, np.float32)
    kind = 0 if deform is None else deform.kind
    coef = np.ascontiguousarray(deform.coef() if deform is not None and kind else [0.0], np.float64)
    vmax = float(255 if bytes_per_voxel == 1 else 65535) if vmax is None else float(vmax)
    nx, ny, nz = shape_xyz
    _check(_lib.dvc_gpu_synth_volume(C.c_void_p(_dev_ptr(vol_dev)), nx, ny, nz, bytes_per_voxel,
                                     len(b), b.ctypes.data_as(C.POINTER(C.c_float)), kind,
                                     _p(coef, _dp), background, noise_sigma, noise_seed, vmax,
                                     C.c_void_p(stream)))


__all__ = ["Engine", "Plan", "Cnn", "read_mhd", "load_raw", "objective", "strain", "order_neighbours", "synth_volume_device", "make_params", "load",
           "DvcError", "E_ARG", "SEED_NEIGHBOURS", "SEED_GIVEN", "SEED_RIGID", "SEED_PARAMS"]
