"""Synthetic speckle volumes, ROI point clouds and `dvc` input files.

No public dataset is used anywhere in this project: every volume is a seeded
synthetic speckle pattern (Gaussian blobs plus Gaussian noise), and the
correlate volume is the same blob field rendered at the inverse-deformed
position of each voxel, with fresh noise. The displacement convention is the
reference's `.disp` one: u = target position - reference position
(Core/InputRead.cpp `print_manual_output`).

This module is the small-volume (numpy, CPU) generator used by tests. Large
benchmark volumes use the device generator `dvc_gpu_synth_volume` in
libdvcgpu.so, which follows the same definition.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np


# --------------------------------------------------------------- deformations
@dataclass
class Affine:
    """u(X) = t + E (X - c)."""
    t: tuple = (0.0, 0.0, 0.0)
    E: tuple = ((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 0.0))
    c: tuple = (0.0, 0.0, 0.0)

    def u(self, X):
        X = np.asarray(X, dtype=np.float64)
        return np.asarray(self.t) + (X - np.asarray(self.c)) @ np.asarray(self.E).T

    def inverse(self, x):
        """X with X + u(X) = x."""
        A = np.eye(3) + np.asarray(self.E)
        rhs = np.asarray(x, np.float64) - np.asarray(self.t) - np.asarray(self.c)
        return np.asarray(self.c) + rhs @ np.linalg.inv(A).T

    def coef(self):
        return [*self.t, *np.asarray(self.E).ravel(), *self.c]

    kind = 1


@dataclass
class Sinusoid:
    """u_i(X) = A sin(2 pi X_j / L) with j = (i+1) mod 3."""
    A: float = 3.0
    L: float = 400.0

    def u(self, X):
        X = np.asarray(X, dtype=np.float64)
        return self.A * np.sin(2.0 * np.pi * np.roll(X, -1, axis=-1) / self.L)

    def inverse(self, x, iters: int = 30):
        x = np.asarray(x, np.float64)
        X = x.copy()
        for _ in range(iters):
            X = x - self.u(X)
        return X

    def coef(self):
        return [self.A, self.L]

    kind = 2


@dataclass
class Bumps:
    """u(X) = t + E (X - c) + sum_k a_k exp(-|X - p_k|^2 / (2 s_k^2)): a smooth
    affine field with Gaussian bumps (rows of `bumps`: px, py, pz, s, ax, ay, az)."""
    t: tuple = (0.0, 0.0, 0.0)
    E: tuple = ((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 0.0))
    c: tuple = (0.0, 0.0, 0.0)
    bumps: tuple = ()

    def u(self, X):
        X = np.asarray(X, dtype=np.float64)
        out = np.asarray(self.t) + (X - np.asarray(self.c)) @ np.asarray(self.E).T
        for px, py, pz, s, ax, ay, az in self.bumps:
            d2 = np.sum((X - np.array([px, py, pz])) ** 2, axis=-1)
            out = out + np.exp(-d2 / (2.0 * s * s))[..., None] * np.array([ax, ay, az])
        return out

    def inverse(self, x, iters: int = 12):
        x = np.asarray(x, np.float64)
        X = x.copy()
        for _ in range(iters):
            X = x - self.u(X)
        return X

    def coef(self):
        out = [*self.t, *np.asarray(self.E).ravel(), *self.c, float(len(self.bumps))]
        for b in self.bumps:
            out += list(map(float, b))
        return out

    kind = 3


def random_bumps(shape_xyz, rng, max_disp=10.0, max_strain=0.02, n_bumps=12):
    """A random smooth field with |u| <= max_disp and |grad u| <~ max_strain:
    a translation, a uniform strain about the centre and Gaussian bumps."""
    c = np.asarray(shape_xyz, np.float64) / 2.0
    E = rng.uniform(-max_strain / 2, max_strain / 2, (3, 3))
    t = rng.uniform(-max_disp / 3, max_disp / 3, 3)
    b = []
    for _ in range(n_bumps):
        s = rng.uniform(48.0, 96.0)
        amp = rng.uniform(-1.0, 1.0, 3) * min(max_disp / 6, max_strain * s)
        b.append((*rng.uniform(0, shape_xyz), s, *amp))
    return Bumps(t=tuple(t), E=tuple(map(tuple, E)), c=tuple(c), bumps=tuple(b))


@dataclass
class Piecewise:
    """Two affine fields split by the plane X_x = split (reference positions):
    u = t1 + E1 (X - c1) where X_x < split, else t2 + E2 (X - c2). The field
    jumps across the plane."""
    t1: tuple = (0.0, 0.0, 0.0)
    E1: tuple = ((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 0.0))
    c1: tuple = (0.0, 0.0, 0.0)
    t2: tuple = (0.0, 0.0, 0.0)
    E2: tuple = ((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 0.0))
    c2: tuple = (0.0, 0.0, 0.0)
    split: float = 0.0

    def _pieces(self):
        return Affine(self.t1, self.E1, self.c1), Affine(self.t2, self.E2, self.c2)

    def u(self, X):
        X = np.asarray(X, dtype=np.float64)
        a, b = self._pieces()
        left = (X[..., 0] < self.split)[..., None]
        return np.where(left, a.u(X), b.u(X))

    def inverse(self, x):
        """Piece 1's inverse where it lands left of the plane, else piece 2's
        (the device renderer's rule)."""
        a, b = self._pieces()
        X1 = a.inverse(x)
        return np.where((X1[..., 0] < self.split)[..., None], X1, b.inverse(x))

    def coef(self):
        return [*self.t1, *np.asarray(self.E1).ravel(), *self.c1, *self.t2, *np.asarray(self.E2).ravel(),
                *self.c2, float(self.split)]

    kind = 4


@dataclass
class BendJump:
    """A smooth bending plus a smoothed planar jump:
    u_x = (J / 2) tanh((X_z - z0) / w), u_y = 0,
    u_z = (kappa / 2) ((X_x - xc)^2 - h)
    (curvature kappa of u_z along x, offset h; a jump of J voxels in u_x
    across the plane X_z = z0, smoothed over w voxels)."""
    kappa: float = 1e-4
    xc: float = 0.0
    h: float = 0.0
    J: float = 2.0
    z0: float = 0.0
    w: float = 5.0

    def u(self, X):
        X = np.asarray(X, dtype=np.float64)
        out = np.zeros_like(X)
        out[..., 0] = 0.5 * self.J * np.tanh((X[..., 2] - self.z0) / self.w)
        out[..., 2] = 0.5 * self.kappa * ((X[..., 0] - self.xc) ** 2 - self.h)
        return out

    def inverse(self, x, iters: int = 20):
        x = np.asarray(x, np.float64)
        X = x.copy()
        for _ in range(iters):
            X = x - self.u(X)
        return X

    def coef(self):
        return [self.kappa, self.xc, self.h, self.J, self.z0, self.w]

    kind = 5


def rotation_z(deg):
    """R - I for a rotation by `deg` degrees about the z axis."""
    th = math.radians(deg)
    c, s = math.cos(th), math.sin(th)
    return ((c - 1.0, -s, 0.0), (s, c - 1.0, 0.0), (0.0, 0.0, 0.0))


@dataclass
class Identity:
    def u(self, X):
        return np.zeros_like(np.asarray(X, np.float64))

    def inverse(self, x):
        return np.asarray(x, np.float64)

    def coef(self):
        return []

    kind = 0


# ----------------------------------------------------------------- speckle ---
def blobs(shape_xyz, n_blobs, sigma=(1.5, 3.0), amp=(40.0, 200.0), seed=1):
    """Random blob list [n, 5]: x, y, z, sigma, amplitude (float64)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape_xyz
    b = np.empty((n_blobs, 5))
    b[:, 0] = rng.uniform(0, nx, n_blobs)
    b[:, 1] = rng.uniform(0, ny, n_blobs)
    b[:, 2] = rng.uniform(0, nz, n_blobs)
    b[:, 3] = rng.uniform(*sigma, n_blobs)
    b[:, 4] = rng.uniform(*amp, n_blobs)
    return b


def render(shape_xyz, blob_list, deform=None, noise_sigma=2.0, noise_seed=2, background=0.0,
           dtype=np.uint8, vmax=None, reach=4.0):
    """Volume [z, y, x] of the blob field at the inverse-deformed voxel positions.

    Each blob contributes amp * exp(-|X(x) - b|^2 / (2 sigma^2)) within `reach`
    sigmas, X(x) the reference position of voxel x. Noise N(0, noise_sigma) is
    added, then the field is rounded and clipped to [0, vmax].
    """
    deform = deform or Identity()
    nx, ny, nz = shape_xyz
    field = np.full((nz, ny, nx), background, dtype=np.float64)
    for bx, by, bz, s, a in blob_list:
        # the blob's image under the field (under each piece of a split field)
        X0 = np.array([bx, by, bz], np.float64)
        fields = deform._pieces() if isinstance(deform, Piecewise) else (deform,)
        img = np.array([X0 + f.u(X0) for f in fields])
        r = reach * s * 1.1 + 1.0
        lo = np.maximum(np.floor(img.min(0) - r).astype(int), 0)
        hi = np.minimum(np.ceil(img.max(0) + r).astype(int) + 1, [nx, ny, nz])
        if np.any(hi <= lo):
            continue
        zz, yy, xx = np.meshgrid(np.arange(lo[2], hi[2]), np.arange(lo[1], hi[1]),
                                 np.arange(lo[0], hi[0]), indexing="ij")
        x = np.stack([xx, yy, zz], axis=-1).astype(np.float64)
        X = deform.inverse(x)
        d2 = np.sum((X - np.array([bx, by, bz])) ** 2, axis=-1)
        w = np.where(d2 <= (reach * s) ** 2, a * np.exp(-d2 / (2 * s * s)), 0.0)
        field[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] += w
    if noise_sigma > 0:
        rng = np.random.default_rng(noise_seed)
        field += rng.normal(0.0, noise_sigma, field.shape)
    if vmax is None:
        vmax = float(np.iinfo(dtype).max)
    return np.clip(np.rint(field), 0, vmax).astype(dtype)


def grid_points(n_xyz, spacing, centre):
    """Regular grid, x fastest; returns [N,3] float64."""
    nx, ny, nz = n_xyz
    off = [(np.arange(m) - (m - 1) / 2.0) * spacing for m in (nx, ny, nz)]
    zz, yy, xx = np.meshgrid(off[2] + centre[2], off[1] + centre[1], off[0] + centre[0],
                             indexing="ij")
    return np.stack([xx.ravel(), yy.ravel(), zz.ravel()], axis=1)


# -------------------------------------------------------------------- files ---
def write_raw(path, vol, header_bytes=0, big_endian=False):
    with open(path, "wb") as f:
        f.write(b"\0" * header_bytes)
        v = vol
        if vol.dtype == np.uint16 and big_endian:
            v = vol.astype(">u2")
        f.write(np.ascontiguousarray(v).tobytes())


def write_roi(path, pts, labels=None):
    labels = np.arange(1, len(pts) + 1) if labels is None else labels
    with open(path, "w") as f:
        for lab, p in zip(labels, pts):
            f.write(f"{int(lab)}\t{p[0]:.3f}\t{p[1]:.3f}\t{p[2]:.3f}\n")


@dataclass
class RunSpec:
    """The `dvc` input-file keys (Core/InputRead.cpp:123-455)."""
    reference_filename: str
    correlate_filename: str
    point_cloud_filename: str
    output_filename: str
    vol_bit_depth: int
    vol_wide: int
    vol_high: int
    vol_tall: int
    subvol_geom: str = "cube"
    subvol_size: int = 31
    subvol_npts: int = 2000
    disp_max: int = 12
    num_srch_dof: int = 6
    obj_function: str = "znssd"
    interp_type: str = "tricubic"
    vol_hdr_lngth: int = 0
    vol_endian: str = "little"
    basin_radius: float = 0.0
    rigid_trans: tuple = (0.0, 0.0, 0.0)
    subvol_aspect: tuple = (1.0, 1.0, 1.0)
    num_points_to_process: int = 0
    starting_point: tuple | None = None
    extra: dict = field(default_factory=dict)

    def write(self, path):
        L = ["# dvc input file (synthetic)",
             f"reference_filename\t{self.reference_filename}\t### reference volume",
             f"correlate_filename\t{self.correlate_filename}\t### correlate volume",
             f"point_cloud_filename\t{self.point_cloud_filename}\t### ROI points",
             f"output_filename\t{self.output_filename}\t### output base",
             f"vol_bit_depth\t{self.vol_bit_depth}"]
        if self.vol_bit_depth != 8:
            L.append(f"vol_endian\t{self.vol_endian}")
        L += [f"vol_hdr_lngth\t{self.vol_hdr_lngth}",
              f"vol_wide\t{self.vol_wide}", f"vol_high\t{self.vol_high}",
              f"vol_tall\t{self.vol_tall}",
              f"subvol_geom\t{self.subvol_geom}", f"subvol_size\t{self.subvol_size}",
              f"subvol_npts\t{self.subvol_npts}", "subvol_thresh\toff",
              f"disp_max\t{self.disp_max}", f"num_srch_dof\t{self.num_srch_dof}",
              f"obj_function\t{self.obj_function}", f"interp_type\t{self.interp_type}",
              "rigid_trans\t{:.6f} {:.6f} {:.6f}".format(*self.rigid_trans),
              f"basin_radius\t{self.basin_radius}",
              "subvol_aspect\t{} {} {}".format(*self.subvol_aspect),
              f"num_points_to_process\t{self.num_points_to_process}"]
        if self.starting_point is not None:
            L.append("starting_point\t{} {} {}".format(*self.starting_point))
        for k, v in self.extra.items():
            L.append(f"{k}\t{v}")
        with open(path, "w") as f:
            f.write("\n".join(L) + "\n")


def cube_subvol_count(npts: int) -> int:
    """Samples of a cube subvolume (Core/Search.cpp:30): ceil(npts^(1/3))^3."""
    return int(math.pow(math.ceil(math.pow(float(npts), 1.0 / 3.0)), 3.0))
