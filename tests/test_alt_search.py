"""The search stages the reference's source holds but never selects.

Search::process_point runs trgrid_global then min_Lev_Mar
(Core/Search.cpp:132,141). Its source also has random_global (:1045-1098),
a coarse stage over random translations from a clock-seeded rand(), and a
Nelder-Mead refinement, look_with(amoeba, ndof, ftol) with min_Nelder_Mead
(:150-181, 379-440, 680-932), which reports Convg_Fail (-2) after 2000
objective evaluations. dvc_params.coarse_method / refine_method select them
here. tests/golden/reference_alt_search.json holds the reference's own
searches with these stages (oracle/_ref drives its Search class through
process_point's steps, its clock fixed at coarse_seed for random_global).

Tolerances: the oracle equals the reference bit for bit. The GPU engine:
statuses identical; with the grid or random translations and Gauss-Newton,
parameters within 1e-3 voxel and objmin within 1e-5 relative, as the other
search tests. Nelder-Mead stops when its vertices' objectives agree to 1e-5
(3 dof) or 1e-7 (6, 12 dof) relative, which is the size of the FP32
evaluation's own error: near the end its comparisons on the GPU and in the
FP64 reference go different ways, and its final vertex agrees only to the
simplex's spread, here within 0.01 voxel, objmin within 1e-3 relative. For
12 dof the reference exhausts its 2000 evaluations (Convg_Fail) where the
GPU's simplex collapses below FP32 resolution and converges, so that case is
pinned through the oracle only.
"""
import json
import os

import numpy as np
import pytest

from fixtures import GOLDEN, SHAPE, hotpath

from digitalvolumecorrelation_gb300.abi import make_params

CASES = json.load(open(os.path.join(GOLDEN, "reference_alt_search.json")))
IDS = [f"{c['volumes']}-{c['params']['num_srch_dof']}dof-{c['params'].get('coarse_method', 'grid')}-"
       f"{c['params'].get('refine_method', 'gauss_newton')}" for c in CASES]


def params_of(case):
    d = hotpath()
    bpv = d[f"vol_{case['volumes']}_ref"].dtype.itemsize
    return make_params(SHAPE, bytes_per_voxel=bpv, interp_type="tricubic", **case["params"])


def test_every_stage_and_status_is_covered():
    kinds = {(c["params"].get("coarse_method", "grid"), c["params"].get("refine_method", "gauss_newton"))
             for c in CASES}
    assert ("grid", "nelder_mead") in kinds and ("random", "gauss_newton") in kinds
    assert ("random", "nelder_mead") in kinds
    st = np.concatenate([c["status"] for c in CASES])
    assert (st == 0).sum() >= 100 and (st == -2).sum() >= 3


@pytest.mark.parametrize("k", range(len(CASES)), ids=IDS)
def test_oracle_vs_reference(oracle, k):
    """The FP64 restatement of both stages equals the reference bit for bit."""
    c = CASES[k]
    d = hotpath()
    vs = c["volumes"]
    o = oracle.process(params_of(c), d[f"vol_{vs}_ref"], d[f"vol_{vs}_cor"], d["search_points"],
                       order=d["search_order"], neigh=d["search_neigh"])
    np.testing.assert_array_equal(o["status"], c["status"])
    np.testing.assert_array_equal(o["params"], np.array(c["params_out"]))
    np.testing.assert_array_equal(o["objmin"], np.array(c["objmin"]))


def test_random_draws_are_the_c_library_generator():
    """random_global's translations: rand() after srand(seed), 2 * rand() an
    int product that wraps, each component in [-disp_max, disp_max)."""
    import ctypes
    libc = ctypes.CDLL(None)
    libc.srand(7)
    draws = np.array([libc.rand() for _ in range(3 * 27)], np.int64)
    twice = ((2 * draws + 2 ** 31) % 2 ** 32) - 2 ** 31
    rel = 3.0 * (twice / 2147483647.0)
    assert rel.min() >= -3.0 - 1e-9 and rel.max() < 3.0 and rel.min() < -1.0 and rel.max() > 1.0


GPU_CASES = [k for k, c in enumerate(CASES)
             if not (c["params"].get("refine_method") == "nelder_mead" and c["params"]["num_srch_dof"] == 12)]


@pytest.mark.gpu
@pytest.mark.parametrize("k", GPU_CASES, ids=[IDS[k] for k in GPU_CASES])
def test_search_vs_reference(gpu_lib, k):
    from digitalvolumecorrelation_gb300 import engine
    c = CASES[k]
    nm = c["params"].get("refine_method") == "nelder_mead"
    tol_p, tol_o = (1e-2, 1e-3) if nm else (1e-3, 1e-5)
    d = hotpath()
    vs = c["volumes"]
    E = engine.Engine(params_of(c), d[f"vol_{vs}_ref"], d[f"vol_{vs}_cor"])
    r = E.process(d["search_points"], order=d["search_order"], neigh=d["search_neigh"])
    st = np.array(c["status"])
    np.testing.assert_array_equal(r["status"], st)
    good = st == 0
    ndof = c["params"]["num_srch_dof"]
    if good.any():
        gp = np.array(c["params_out"])
        dp = np.abs(r["params"][good, :ndof] - gp[good, :ndof])
        assert dp.max() <= tol_p, dp.max()
        ro = np.array(c["objmin"])[good]
        rel = np.abs(r["objmin"][good] - ro) / np.abs(ro)
        assert rel.max() <= tol_o, rel.max()
    assert np.all(r["params"][~good] == 0.0)
    E.close()
