"""Known answers of the interpolation and the search, for the FP64 oracle and
for the reference's own code where it is built here (oracle/_ref).

The reference's tests pin no numerical result of its hot path; these follow
from the mathematics of the method:
  * tricubic (Lekien-Marsden over central finite differences) reproduces
    every polynomial of degree <= 2 exactly: its differences are exact for
    such a polynomial, and the cubic Hermite form then is the polynomial;
  * trilinear reproduces every multilinear function (1, x, y, z, xy, yz,
    zx, xyz) exactly;
  * a correlate volume that is the reference volume moved by whole voxels
    is matched exactly: the search returns that translation, no rotation or
    strain, and an objective of zero.
Volumes are stored z, y, x (x fastest); positions are (x, y, z).
"""
import numpy as np
import pytest

from digitalvolumecorrelation_gb300.abi import make_params

N = 30


def _grid():
    Z, Y, X = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    return X.astype(np.float64), Y.astype(np.float64), Z.astype(np.float64)


def quadratic(x, y, z):
    return 1000 + 7 * x + 5 * y + 3 * z + 2 * x * y + x * z + y * z + x * x + 2 * y * y + z * z


def multilinear(x, y, z):
    return 1000 + 3 * x + 2 * y + z + x * y + x * z + y * z + x * y * z


CASES = [("tricubic", 2, quadratic), ("trilinear", 1, multilinear)]


def _interp_case(fn):
    X, Y, Z = _grid()
    vol = fn(X, Y, Z)
    assert vol.max() < 65535
    vol = vol.astype(np.uint16)
    p = make_params((N, N, N), bytes_per_voxel=2, subvol_size=11, subvol_npts=300, disp_max=3)
    center = np.array([15.0, 15.0, 15.0])
    pts = center + np.random.default_rng(4).uniform(-4.0, 4.0, (300, 3))
    return p, vol, center, pts, fn(pts[:, 0], pts[:, 1], pts[:, 2])


@pytest.mark.parametrize("name,it,fn", CASES, ids=[c[0] for c in CASES])
def test_interpolation_reproduces_polynomials_oracle(oracle, name, it, fn):
    p, vol, center, pts, exact = _interp_case(fn)
    got, undefined = oracle.interpolate(p, vol, center, pts, it)
    assert got is not None and undefined == 0
    assert np.abs(got - exact).max() <= 1e-9 * np.abs(exact).max()


@pytest.mark.parametrize("name,it,fn", CASES, ids=[c[0] for c in CASES])
def test_interpolation_reproduces_polynomials_reference(reference, name, it, fn):
    p, vol, center, pts, exact = _interp_case(fn)
    got = reference.interpolate(p, vol, center, pts, it)
    assert got is not None
    assert np.abs(got - exact).max() <= 1e-9 * np.abs(exact).max()


SHIFT = np.array([2.0, -1.0, 1.0])


def _shift_case(dof, geom):
    from digitalvolumecorrelation_gb300 import synth
    shape = (48, 48, 48)
    b = synth.blobs(shape, 150, seed=71)
    ref = synth.render(shape, b, noise_sigma=2.0, noise_seed=72)
    # cor(X + u) = ref(X) for the whole-voxel translation u (x, y, z)
    cor = np.roll(ref, shift=(int(SHIFT[2]), int(SHIFT[1]), int(SHIFT[0])), axis=(0, 1, 2))
    p = make_params(shape, subvol_geom=geom, subvol_size=11, subvol_npts=400, num_srch_dof=dof, disp_max=4,
                    basin_radius=0.0, rigid_trans=tuple(SHIFT + [0.3, -0.2, 0.4]))
    pts = synth.grid_points((2, 2, 2), 6.0, (24.0, 24.0, 24.0))
    return p, ref, cor, pts


def _check_shift(r, dof):
    assert np.all(r["status"] == 0), r["status"]
    assert np.abs(r["params"][:, :3] - SHIFT).max() <= 1e-6
    if dof > 3:
        assert np.abs(r["params"][:, 3:dof]).max() <= 1e-6
    assert np.abs(r["objmin"]).max() <= 1e-10


@pytest.mark.parametrize("dof,geom", [(3, "cube"), (6, "sphere"), (12, "cube")])
def test_whole_voxel_translation_found_exactly_oracle(oracle, dof, geom):
    p, ref, cor, pts = _shift_case(dof, geom)
    order, neigh = oracle.order_neighbours(pts)
    _check_shift(oracle.process(p, ref, cor, pts, order=order, neigh=neigh), dof)


@pytest.mark.parametrize("dof,geom", [(3, "cube"), (6, "sphere"), (12, "cube")])
def test_whole_voxel_translation_found_exactly_reference(oracle, reference, dof, geom):
    p, ref, cor, pts = _shift_case(dof, geom)
    order, neigh = oracle.order_neighbours(pts)
    _check_shift(reference.process(p, ref, cor, pts, order, neigh), dof)
