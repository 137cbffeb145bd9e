"""The benchmark and parity workloads, as synthetic data of the named shapes.

No public dataset exists for this path; each workload is a seeded synthetic
speckle pair with the sizes, value ranges and deformations of the named
configuration. Volumes are rendered on the GPU by `dvc_gpu_synth_volume`
(or, for small CPU tests, by synth.render).

  config 1 ("plain"): 256^3 uint8, 1500 blobs (sigma 1.5-3, amplitude 40-200),
      noise sigma 2; target = translation (2.3, -1.7, 0.6) + 0.5% uniform
      strain about the centre; 10^3 ROI grid, spacing 12, centred; cube 31 /
      2000 samples, znssd, tricubic, 6 dof, basin_radius 6, disp_max 12.
  config 2 ("precision + scale"): 1024^3 uint16, blobs with amplitude
      2000-60000 at one blob per 1000 voxels (density chosen here: the
      configuration leaves it open), noise sigma 150; u_i = 3 sin(2 pi X_j/400);
      40 x 40 x 38 = 60,800-point grid (spacing 24); sphere of diameter 41 /
      4000 samples, znssd, tricubic, 12 dof; disp_max 6 and basin_radius 3
      (chosen here: the configuration leaves them open).
  config 3 ("batching, uneven workload"): 768^3 uint8, one blob per 1000
      voxels (sigma 1.5-3, amplitude 40-200), noise sigma 2; target = a split
      field: left of x = 384 a rigid rotation of 1.5 degrees about the z axis
      through (192, 384, 384) plus a translation (1, -0.5, 0.5), right of it
      1% uniaxial compression along z about z = 384; 40,000 ROI points at
      uniform random positions (64 voxels from the faces; the first at the
      rotation centre, where the processing order starts), each point its own
      configuration: subvol_size from {21, 31, 41, 61, 81}, cube or sphere,
      subvol_npts = 0.15 x the subvolume's voxel count (at most the
      reference's 50,000), 3, 6 or 12 dof, ssd or znssd; tricubic, disp_max 8
      and basin_radius 4 (chosen here); strain window 7.
  config 5 ("full pipeline, large"): 2048 x 2048 x 1024 uint16 (8 GiB pair),
      blobs as config 2; target = a smooth bending u_z = (1e-4 / 2)((x -
      1024)^2 - 395^2 / 2) (curvature 1e-4 per voxel, |u_z| <= 3.9 over the
      ROI) plus a 2-voxel jump of u_x across z = 512 smoothed over 5 voxels
      (u_x = tanh((z - 512) / 5)); 80 x 80 x 78 = 499,200-point grid of
      spacing 10 centred at (1024, 1024, 512); cube 41 / 3000 samples (15^3 =
      3375), znssd, tricubic, 12 dof, disp_max 6 and basin_radius 3 (chosen
      here); learned start with the plain search as fallback where the
      refined ZNSSD exceeds 0.1; strain window 5.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import synth
from .abi import make_params


@dataclass
class Workload:
    name: str
    shape: tuple
    bytes_per_voxel: int
    params_kw: dict
    points: np.ndarray
    deform: object
    blobs: np.ndarray
    noise_sigma: float
    ref_seed: int
    cor_seed: int

    def params(self):
        return make_params(self.shape, bytes_per_voxel=self.bytes_per_voxel, **self.params_kw)

    def truth(self, pts=None):
        """True displacement u(X) at the ROI points (target - reference)."""
        return self.deform.u(self.points if pts is None else pts)

    @property
    def nvox(self):
        return int(np.prod(self.shape))

    def render_device(self, torch_device="cuda"):
        """Both volumes as uint8/int16-storage torch tensors on the GPU."""
        import torch
        from .engine import synth_volume_device
        dt = torch.uint8 if self.bytes_per_voxel == 1 else torch.int16
        # +64 bytes of tail padding (the engine reads whole aligned words)
        pad = 64 // self.bytes_per_voxel
        ref = torch.zeros(self.nvox + pad, dtype=dt, device=torch_device)
        cor = torch.zeros(self.nvox + pad, dtype=dt, device=torch_device)
        vmax = 255.0 if self.bytes_per_voxel == 1 else 65535.0
        synth_volume_device(ref, self.shape, self.bytes_per_voxel, self.blobs, None, 0.0,
                            self.noise_sigma, self.ref_seed, vmax)
        synth_volume_device(cor, self.shape, self.bytes_per_voxel, self.blobs, self.deform, 0.0,
                            self.noise_sigma, self.cor_seed, vmax)
        torch.cuda.synchronize()
        return ref, cor


def config1(n_points_axis=10):
    shape = (256, 256, 256)
    c = (128.0, 128.0, 128.0)
    deform = synth.Affine(t=(2.3, -1.7, 0.6),
                          E=((0.005, 0, 0), (0, 0.005, 0), (0, 0, 0.005)), c=c)
    pts = synth.grid_points((n_points_axis,) * 3, 12.0, c)
    kw = dict(subvol_geom="cube", subvol_size=31, subvol_npts=2000, obj_function="znssd",
              interp_type="tricubic", num_srch_dof=6, disp_max=12, basin_radius=6.0)
    b = synth.blobs(shape, 1500, sigma=(1.5, 3.0), amp=(40.0, 200.0), seed=1)
    return Workload("config1_256cube_u8_1000pts_cube31_dof6", shape, 1, kw, pts, deform, b, 2.0,
                    101, 102)


def config2(grid=(40, 40, 38), spacing=24.0):
    shape = (1024, 1024, 1024)
    c = (512.0, 512.0, 512.0)
    deform = synth.Sinusoid(A=3.0, L=400.0)
    pts = synth.grid_points(grid, spacing, c)
    kw = dict(subvol_geom="sphere", subvol_size=41, subvol_npts=4000, obj_function="znssd",
              interp_type="tricubic", num_srch_dof=12, disp_max=6, basin_radius=3.0)
    n_blobs = int(np.prod(shape) // 1000)
    b = synth.blobs(shape, n_blobs, sigma=(1.5, 3.0), amp=(2000.0, 60000.0), seed=2)
    return Workload("config2_1024cube_u16_60800pts_sphere41_dof12", shape, 2, kw, pts, deform, b,
                    150.0, 201, 202)


CONFIG3_SIZES = (21, 31, 41, 61, 81)
CONFIG3_GEOMS = ("cube", "sphere")
CONFIG3_DOFS = (3, 6, 12)
CONFIG3_OBJS = ("ssd", "znssd")


def config3_settings():
    """The 60 search configurations of configuration 3, index
    ((size * 2 + geom) * 3 + dof) * 2 + objective."""
    out = []
    for size in CONFIG3_SIZES:
        for geom in CONFIG3_GEOMS:
            vox = size ** 3 if geom == "cube" else 4.0 / 3.0 * np.pi * (size / 2.0) ** 3
            npts = int(min(50000, round(0.15 * vox)))
            for dof in CONFIG3_DOFS:
                for obj in CONFIG3_OBJS:
                    out.append(dict(subvol_geom=geom, subvol_size=size, subvol_npts=npts, obj_function=obj,
                                    interp_type="tricubic", num_srch_dof=dof, disp_max=8, basin_radius=4.0))
    return out


def config3(n_points=40000, shape=(768, 768, 768), seed=3):
    """Returns (workload, per-point configuration index, configuration list);
    the workload's params_kw is the first configuration's (volumes only)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    split = nx / 2.0
    rc = (nx / 4.0, ny / 2.0, nz / 2.0)
    deform = synth.Piecewise(t1=(1.0, -0.5, 0.5), E1=synth.rotation_z(1.5), c1=rc,
                             t2=(0.0, 0.0, 0.0), E2=((0, 0, 0), (0, 0, 0), (0, 0, -0.01)),
                             c2=(nx / 2.0, ny / 2.0, nz / 2.0), split=split)
    margin = 64.0
    pts = rng.uniform(margin, np.array(shape, np.float64) - margin, (n_points, 3))
    pts[0] = rc
    settings = config3_settings()
    cfg = rng.integers(0, len(settings), n_points).astype(np.int32)
    n_blobs = int(np.prod(shape) // 1000)
    b = synth.blobs(shape, n_blobs, sigma=(1.5, 3.0), amp=(40.0, 200.0), seed=seed + 30)
    W = Workload("config3_768cube_u8_40000pts_mixed60", shape, 1, settings[0], pts, deform, b, 2.0,
                 seed + 301, seed + 302)
    return W, cfg, settings


def config5(grid=(80, 80, 78), spacing=10.0, shape=(2048, 2048, 1024)):
    nx, ny, nz = shape
    c = (nx / 2.0, ny / 2.0, nz / 2.0)
    half = (grid[0] - 1) * spacing / 2.0
    deform = synth.BendJump(kappa=1e-4, xc=c[0], h=half * half / 2.0, J=2.0, z0=c[2], w=5.0)
    pts = synth.grid_points(grid, spacing, c)
    kw = dict(subvol_geom="cube", subvol_size=41, subvol_npts=3000, obj_function="znssd",
              interp_type="tricubic", num_srch_dof=12, disp_max=6, basin_radius=3.0)
    n_blobs = int(np.prod(shape) // 1000)
    b = synth.blobs(shape, n_blobs, sigma=(1.5, 3.0), amp=(2000.0, 60000.0), seed=5)
    return Workload("config5_2048x2048x1024_u16_499200pts_cube41_dof12", shape, 2, kw, pts, deform, b,
                    150.0, 501, 502)


def order_and_neighbours(points, n_neigh=75, start=None):
    """Processing order by distance from the start point and the n_neigh
    nearest points of each point (DataCloud::sort_order_neighbors,
    Core/DataCloud.cpp:69-144): stable sorts on exact distances, so the order
    among equidistant points is by index. The reference's std::sort leaves
    that order to its implementation; the `dvc` host program uses std::sort
    itself where the exact reference order matters."""
    from scipy.spatial import cKDTree
    pts = np.asarray(points, np.float64)
    s = pts[0] if start is None else np.asarray(start, np.float64)
    d0 = np.sqrt(((pts - s) ** 2).sum(1))
    order = np.argsort(d0, kind="stable").astype(np.int32)
    k = min(n_neigh, len(pts))
    tree = cKDTree(pts)
    # query a few extra candidates, then order them by exact distance and index
    kk = min(len(pts), k + 16)
    dist, idx = tree.query(pts, k=kk)
    neigh = np.empty((len(pts), k), np.int32)
    for i in range(len(pts)):
        cand = idx[i]
        dd = np.sqrt(((pts[cand] - pts[i]) ** 2).sum(1))
        o = np.lexsort((cand, dd))
        neigh[i] = cand[o[:k]]
    return order, neigh
