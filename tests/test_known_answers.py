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
    strain, and an objective of zero;
  * the strain fit of a displacement field linear in the position recovers
    its gradient, hence both strain measures and their principal values;
  * each objective is zero for identical signals and blind exactly to what
    its normalisation removes (offset, scale);
  * Nelder-Mead and random_global followed by Gauss-Newton find the
    whole-voxel translation too.
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


# ----------------------------------------------------------------- strain ---
# A displacement field linear in the position, u = A X + b: every strain
# window's least-squares fit recovers the displacement gradient A and the
# displacement itself exactly, so the engineering strain is (A + A')/2 and
# the Lagrangian strain (A + A' + A'A)/2, each with its eigenvalues in
# descending order. Integer grid positions and A, b in multiples of 1e-3 keep
# u exact in the .disp file's six decimals.
A_LIN = np.array([[0.010, 0.002, -0.003], [0.001, -0.006, 0.004], [0.002, 0.003, 0.008]])
B_LIN = np.array([1.5, -0.7, 0.3])


def _linear_field():
    from digitalvolumecorrelation_gb300 import synth
    pts = synth.grid_points((6, 6, 6), 8.0, (48.0, 48.0, 48.0))
    assert np.all(pts == np.round(pts))
    return pts, pts @ A_LIN.T + B_LIN


def _strain_rows(S):
    comps = [S[0, 0], S[1, 1], S[2, 2], S[0, 1], S[1, 2], S[0, 2]]
    return np.array(comps + sorted(np.linalg.eigvalsh(S), reverse=True))


E_LIN = _strain_rows(0.5 * (A_LIN + A_LIN.T))
L_LIN = _strain_rows(0.5 * (A_LIN + A_LIN.T + A_LIN.T @ A_LIN))


@pytest.mark.parametrize("ndp,refill", [(25, False), (25, True), (60, False)])
def test_strain_of_a_linear_field_oracle(oracle, ndp, refill):
    """(Windows of about 10 points on this lattice can be rank-deficient,
    where no fit recovers A: 25 is the reference's default.)"""
    pts, disp = _linear_field()
    n = len(pts)
    _, neigh = oracle.order_neighbours(pts)
    r = oracle.strain(pts, np.zeros(n, np.int32), np.full(n, 0.01), disp, neigh, ndp, 1.0, refill)
    assert np.abs(r["dgrad"] - A_LIN.ravel()).max() <= 1e-12
    assert np.abs(r["u_fit"] - disp).max() <= 1e-10
    assert np.abs(r["e_strain"] - E_LIN).max() <= 1e-12
    assert np.abs(r["l_strain"] - L_LIN).max() <= 1e-12


def test_strain_of_a_linear_field_reference_program(tmp_path):
    """The reference's own `strain` program (oracle/_ref) on the same field
    written as a .disp file: its Lagrangian, engineering and gradient CSVs
    carry the exact values to their six printed digits."""
    import os
    import subprocess
    exe = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "strain")
    if not os.path.exists(exe):
        pytest.skip("the reference's strain is built only where its sources are (oracle/build_ref.sh)")
    pts, disp = _linear_field()
    with open(os.path.join(str(tmp_path), "lin.disp"), "w") as f:
        f.write("n\tx\ty\tz\tstatus\tobjmin\tu\tv\tw\n")
        for k, (p, u) in enumerate(zip(pts, disp)):
            f.write(f"{k + 1}\t{p[0]:g}\t{p[1]:g}\t{p[2]:g}\t0\t0.01\t{u[0]:.6f}\t{u[1]:.6f}\t{u[2]:.6f}\n")
    r = subprocess.run([exe, "lin.disp", "-E", "-D"], cwd=str(tmp_path), capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr

    def rows(name):
        lines = open(os.path.join(str(tmp_path), name)).read().strip().split("\n")[1:]
        return np.array([[float(v) for v in l.split(",")] for l in lines])

    def sig6(actual, printed):
        mag = np.where(printed == 0, 1e-300, np.abs(printed))
        tol = np.maximum(0.5001 * 10.0 ** (np.floor(np.log10(mag)) - 5), 1e-12)
        assert np.all(np.abs(actual - printed) <= tol), np.max(np.abs(actual - printed) / tol)
    Lr, Er, Dr = rows("lin-sw25.Lstr.csv"), rows("lin-sw25.Estr.csv"), rows("lin-sw25.dgrd.csv")
    assert len(Lr) == len(pts)
    sig6(np.broadcast_to(L_LIN, Lr[:, 9:18].shape), Lr[:, 9:18])
    sig6(np.broadcast_to(E_LIN, Er[:, 9:18].shape), Er[:, 9:18])
    sig6(np.broadcast_to(A_LIN.ravel(), Dr[:, 9:18].shape), Dr[:, 9:18])


# -------------------------------------------------------------- objectives ---
# What each objective's definition (Core/ObjectiveFunctions.cpp:24-263)
# makes it blind to: ZSSD to an offset of the target, NSSD to a positive
# scale, ZNSSD to both; every objective is zero for identical signals.
OBJ = {"sad": 0, "ssd": 1, "zssd": 2, "nssd": 3, "znssd": 4}
INVARIANT = {"zssd": [(1.0, 30.0)], "nssd": [(2.5, 0.0)], "znssd": [(2.5, 0.0), (1.0, 30.0), (0.4, -3.0)]}


def _signals():
    rng = np.random.default_rng(3)
    r = rng.uniform(10.0, 200.0, 500)
    return r, r + rng.normal(0.0, 5.0, 500)


def _check_objective(obj, name):
    r, t = _signals()
    f = OBJ[name]
    base = obj(f, r, t)
    assert base > 0.0
    assert abs(obj(f, r, r)) <= 1e-12 * max(1.0, abs(base))
    for a, b in INVARIANT.get(name, []):
        assert abs(obj(f, r, a * t + b) - base) <= 1e-12 * abs(base), (name, a, b)
    # and not blind to what its definition does not remove
    if name in ("sad", "ssd", "nssd"):
        assert abs(obj(f, r, t + 30.0) - base) > 1e-3 * abs(base)
    if name in ("sad", "ssd", "zssd"):
        assert abs(obj(f, r, 2.5 * t) - base) > 1e-3 * abs(base)


@pytest.mark.parametrize("name", list(OBJ))
def test_objective_invariances_oracle(oracle, name):
    _check_objective(oracle.objective, name)


@pytest.mark.parametrize("name", list(OBJ))
def test_objective_invariances_reference(reference, name):
    _check_objective(reference.objective, name)


# The search stages the reference's source holds but never selects
# (Core/Search.cpp:150-181, 379-440, 680-932, 1045-1098) meet the same answer:
# Nelder-Mead from the start, and random_global's translations before
# Gauss-Newton, find the whole-voxel translation with a zero objective.
STAGES = [("nelder_mead", 3, "cube", dict(refine_method="nelder_mead")),
          ("nelder_mead", 6, "sphere", dict(refine_method="nelder_mead")),
          ("random_global", 6, "cube", dict(coarse_method="random", coarse_seed=11, basin_radius=2.0))]


def _stage_case(dof, geom, kw):
    p, ref, cor, pts = _shift_case(dof, geom)
    q = make_params(ref.shape, subvol_geom=geom, subvol_size=11, subvol_npts=400, num_srch_dof=dof, disp_max=4,
                    rigid_trans=tuple(SHIFT + [0.3, -0.2, 0.4]), **dict(dict(basin_radius=0.0), **kw))
    return q, ref, cor, pts


def _check_stage(r, tol_u, tol_obj):
    assert np.all(r["status"] == 0), r["status"]
    assert np.abs(r["params"][:, :3] - SHIFT).max() <= tol_u
    assert np.abs(r["objmin"]).max() <= tol_obj


@pytest.mark.parametrize("stage,dof,geom,kw", STAGES, ids=[f"{s[0]}-{s[1]}" for s in STAGES])
def test_search_stages_find_whole_voxel_translation(oracle, reference, stage, dof, geom, kw):
    p, ref, cor, pts = _stage_case(dof, geom, kw)
    order, neigh = oracle.order_neighbours(pts)
    o = oracle.process(p, ref, cor, pts, order=order, neigh=neigh)
    r = reference.process_stages(p, ref, cor, pts, order, neigh)
    # Gauss-Newton from a random translation up to disp_max away stops by
    # its rule (update below 0.01 voxel) a few millionths of a voxel short
    tol_u, tol_obj = (1e-6, 1e-10) if stage == "nelder_mead" else (1e-4, 1e-8)
    _check_stage(o, tol_u, tol_obj)
    _check_stage(r, tol_u, tol_obj)
    np.testing.assert_array_equal(o["status"], r["status"])
    assert np.abs(o["params"] - r["params"]).max() <= 1e-9
