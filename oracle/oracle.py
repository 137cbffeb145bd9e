"""ctypes access to the CPU oracles. TEST INFRASTRUCTURE ONLY.

Two checkers live under oracle/:
  * liboracle.so  — dvc_oracle.cpp, the FP64 restatement of the reference's
                    hot path (builds on any host with g++);
  * _ref/libdvcref.so — the reference's own Core/*.cpp compiled by
                    build_ref.sh (only where the reference sources exist).
Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg import
this module. The product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

from digitalvolumecorrelation_gb300.abi import DvcParams, E_RANGE

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libdvcref.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build_oracle(force=False):
    """Compile dvc_oracle.cpp (portable C++, no GPU needed)."""
    src = os.path.join(HERE, "dvc_oracle.cpp")
    if not force and os.path.exists(ORACLE_SO) and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src):
        return ORACLE_SO
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    subprocess.check_call(["g++", "-std=c++17", "-O3", "-fopenmp", "-fPIC", "-ffp-contract=off",
                           "-shared", "-o", ORACLE_SO, src])
    return ORACLE_SO


def build_reference():
    """Run oracle/build_ref.sh; returns the .so path or None when the
    reference sources are absent."""
    r = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], capture_output=True, text=True)
    return REF_SO if r.returncode == 0 and os.path.exists(REF_SO) else None


def reference_dir():
    """The reference sources' directory as oracle/build_ref.sh finds it
    (DVC_REFERENCE_DIR or the recipe's default), or None where they are absent."""
    r = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), "--where"], capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 and r.stdout.strip() else None


def _ptr(a, t):
    return a.ctypes.data_as(t)


class Oracle:
    """FP64 restatement (dvc_oracle.cpp)."""

    def __init__(self, path=None):
        self.lib = C.CDLL(path or build_oracle())
        L = self.lib
        L.oracle_process.restype = C.c_int
        L.oracle_interpolate.restype = C.c_int
        L.oracle_objective.restype = C.c_double
        L.oracle_sample_cloud.restype = C.c_int
        L.oracle_order_neighbours.restype = C.c_int
        L.oracle_strain.restype = C.c_int
        L.oracle_lekien_coefficients.restype = C.c_int

    def process(self, p: DvcParams, ref, cor, points, order=None, neigh=None, n_process=None,
                seed_mode=0, seeds=None, n_threads=0):
        pts = np.ascontiguousarray(points, np.float64)
        n = len(pts)
        order = np.arange(n, dtype=np.int32) if order is None else np.ascontiguousarray(order, np.int32)
        n_process = len(order) if n_process is None else n_process
        nn = 0 if neigh is None else neigh.shape[1]
        neigh_a = np.zeros((n, 1), np.int32) if neigh is None else np.ascontiguousarray(neigh, np.int32)
        seeds_a = np.zeros((n, 3)) if seeds is None else np.ascontiguousarray(seeds, np.float64)
        status = np.zeros(n, np.int32)
        objmin = np.zeros(n)
        par = np.zeros((n, 12))
        its = np.zeros(n, np.int32)
        ne = C.c_longlong(0)
        und = C.c_longlong(0)
        ref = np.ascontiguousarray(ref)
        cor = np.ascontiguousarray(cor)
        self.lib.oracle_process(C.byref(p), ref.ctypes.data_as(C.c_void_p),
                                cor.ctypes.data_as(C.c_void_p), n, _ptr(pts, _dp), n_process,
                                _ptr(order, _ip), nn, _ptr(neigh_a, _ip), seed_mode,
                                _ptr(seeds_a, _dp), _ptr(status, _ip), _ptr(objmin, _dp),
                                _ptr(par, _dp), _ptr(its, _ip), C.byref(ne), C.byref(und),
                                int(n_threads))
        return dict(status=status, objmin=objmin, params=par, gn_iters=its,
                    n_evals=ne.value, undefined_evals=und.value)

    def interpolate(self, p: DvcParams, vol, center, pts, interp_type=2):
        pts = np.ascontiguousarray(pts, np.float64)
        out = np.zeros(len(pts))
        und = C.c_longlong(0)
        c = (C.c_double * 3)(*center)
        vol = np.ascontiguousarray(vol)
        rc = self.lib.oracle_interpolate(C.byref(p), vol.ctypes.data_as(C.c_void_p), c, len(pts),
                                         _ptr(pts, _dp), interp_type, _ptr(out, _dp), C.byref(und))
        return (None if rc == E_RANGE else out), und.value

    def objective(self, fcn, ref, tar, residual=False):
        ref = np.ascontiguousarray(ref, np.float64)
        tar = np.ascontiguousarray(tar, np.float64)
        res = np.zeros(len(ref)) if residual else None
        o = self.lib.oracle_objective(fcn, len(ref), _ptr(ref, _dp), _ptr(tar, _dp),
                                      _ptr(res, _dp) if residual else None)
        return (o, res) if residual else o

    def lekien_matrix(self):
        m = np.zeros((64, 64))
        self.lib.oracle_lekien_matrix(_ptr(m, _dp))
        return m

    def lekien_coefficients(self, p, vol, center, cells):
        cells = np.ascontiguousarray(cells, np.int32)
        out = np.zeros((len(cells), 64))
        c = (C.c_double * 3)(*center)
        vol = np.ascontiguousarray(vol)
        rc = self.lib.oracle_lekien_coefficients(C.byref(p), vol.ctypes.data_as(C.c_void_p), c,
                                                 len(cells), _ptr(cells, _ip), _ptr(out, _dp))
        assert rc == 0, rc
        return out

    def sample_cloud(self, p, pt):
        n = self.lib.oracle_sample_cloud(C.byref(p), (C.c_double * 3)(*pt), None)
        out = np.zeros((n, 3))
        self.lib.oracle_sample_cloud(C.byref(p), (C.c_double * 3)(*pt), _ptr(out, _dp))
        return out

    def order_neighbours(self, pts, start=None, n_neigh=75):
        pts = np.ascontiguousarray(pts, np.float64)
        n = len(pts)
        start = pts[0] if start is None else start
        order = np.zeros(n, np.int32)
        keep = min(n_neigh, n)
        neigh = np.zeros((n, keep), np.int32)
        self.lib.oracle_order_neighbours(n, _ptr(pts, _dp), (C.c_double * 3)(*start), n_neigh,
                                         _ptr(order, _ip), _ptr(neigh, _ip))
        return order, neigh

    def strain(self, pts, status, objmin, disp, neigh, ndp=25, objt=1.0, refill=False, planar=0):
        n = len(pts)
        pts = np.ascontiguousarray(pts, np.float64)
        status = np.ascontiguousarray(status, np.int32)
        objmin = np.ascontiguousarray(objmin, np.float64)
        disp = np.ascontiguousarray(disp, np.float64)
        neigh = np.ascontiguousarray(neigh, np.int32)
        out = dict(u_fit=np.zeros((n, 3)), pts_in_sw=np.zeros(n, np.int32), sw_radius=np.zeros(n),
                   e_strain=np.zeros((n, 9)), l_strain=np.zeros((n, 9)), dgrad=np.zeros((n, 9)))
        self.lib.oracle_strain(n, _ptr(pts, _dp), _ptr(status, _ip), _ptr(objmin, _dp),
                               _ptr(disp, _dp), neigh.shape[1], _ptr(neigh, _ip), ndp,
                               C.c_double(objt), int(refill), int(planar),
                               _ptr(out["u_fit"], _dp), _ptr(out["pts_in_sw"], _ip),
                               _ptr(out["sw_radius"], _dp), _ptr(out["e_strain"], _dp),
                               _ptr(out["l_strain"], _dp), _ptr(out["dgrad"], _dp))
        return out


class Reference:
    """The reference's own classes (oracle/_ref/libdvcref.so). Volumes go
    through raw files because the reference reads them from disk."""

    def __init__(self, path=REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.lib.ref_objective.restype = C.c_double
        self.tmp = tempfile.TemporaryDirectory(prefix="dvcref_")

    def _file(self, vol, name):
        path = os.path.join(self.tmp.name, name)
        np.ascontiguousarray(vol).tofile(path)
        return path.encode()

    def interpolate(self, p, vol, center, pts, interp_type=2):
        f = self._file(vol, "vol.raw")
        pts = np.ascontiguousarray(pts, np.float64)
        out = np.zeros(len(pts))
        rc = self.lib.ref_interpolate(C.byref(p), f, 0, b"little", (C.c_double * 3)(*center),
                                      len(pts), _ptr(pts, _dp), interp_type, _ptr(out, _dp))
        return None if rc == E_RANGE else out

    def objective(self, fcn, ref, tar, residual=False):
        ref = np.ascontiguousarray(ref, np.float64)
        tar = np.ascontiguousarray(tar, np.float64)
        res = np.zeros(len(ref))
        o = self.lib.ref_objective(fcn, len(ref), _ptr(ref, _dp), _ptr(tar, _dp), _ptr(res, _dp))
        return (o, res) if residual else o

    def process(self, p, ref, cor, points, order, neigh, n_process=None):
        fr = self._file(ref, "ref.raw")
        fc = self._file(cor, "cor.raw")
        pts = np.ascontiguousarray(points, np.float64)
        n = len(pts)
        order = np.ascontiguousarray(order, np.int32)
        neigh = np.ascontiguousarray(neigh, np.int32)
        n_process = len(order) if n_process is None else n_process
        status = np.zeros(n, np.int32)
        objmin = np.zeros(n)
        par = np.zeros((n, 12))
        self.lib.ref_process(C.byref(p), fr, fc, 0, b"little", n, _ptr(pts, _dp), n_process,
                             _ptr(order, _ip), neigh.shape[1], _ptr(neigh, _ip),
                             _ptr(status, _ip), _ptr(objmin, _dp), _ptr(par, _dp))
        return dict(status=status, objmin=objmin, params=par)

    def process_stages(self, p, ref, cor, points, order, neigh, n_process=None):
        """process() with the search stages p.coarse_method / p.refine_method
        (random_global with its clock fixed at p.coarse_seed; Nelder-Mead)."""
        fr = self._file(ref, "ref.raw")
        fc = self._file(cor, "cor.raw")
        pts = np.ascontiguousarray(points, np.float64)
        n = len(pts)
        order = np.ascontiguousarray(order, np.int32)
        neigh = np.ascontiguousarray(neigh, np.int32)
        n_process = len(order) if n_process is None else n_process
        status = np.zeros(n, np.int32)
        objmin = np.zeros(n)
        par = np.zeros((n, 12))
        self.lib.ref_process_stages(C.byref(p), fr, fc, 0, b"little", n, _ptr(pts, _dp), n_process,
                                    _ptr(order, _ip), neigh.shape[1], _ptr(neigh, _ip),
                                    _ptr(status, _ip), _ptr(objmin, _dp), _ptr(par, _dp))
        return dict(status=status, objmin=objmin, params=par)

    def order_neighbours(self, pts, start=None):
        pts = np.ascontiguousarray(pts, np.float64)
        n = len(pts)
        start = pts[0] if start is None else start
        order = np.zeros(n, np.int32)
        neigh = np.zeros((n, min(75, n)), np.int32)
        self.lib.ref_order_neighbours(n, _ptr(pts, _dp), (C.c_double * 3)(*start),
                                      _ptr(order, _ip), _ptr(neigh, _ip))
        return order, neigh
