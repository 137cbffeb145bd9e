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
