"""Processing order and k-nearest neighbours on the GPU
(dvc_gpu_order_neighbours) against a numpy restatement with the same
distances and the documented tie rule (distance, then index), and against the
reference-order host path (the FP64 oracle's std::sort) up to the order of
tied points."""
from __future__ import annotations

import numpy as np
import pytest


def reference_rule(pts, start, k):
    """numpy: the reference's distance formula, ties by index."""
    def dist(a, b):
        d = a - b
        return np.sqrt((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2])
    d0 = dist(pts, start[None, :])
    order = np.lexsort((np.arange(len(pts)), d0)).astype(np.int32)
    kk = min(k, len(pts))
    neigh = np.zeros((len(pts), kk), np.int32)
    for i in range(len(pts)):
        di = dist(pts, pts[i][None, :])
        neigh[i] = np.lexsort((np.arange(len(pts)), di))[:kk]
    return order, neigh


def clouds():
    from digitalvolumecorrelation_gb300 import synth
    rng = np.random.default_rng(4)
    yield "grid", synth.grid_points((9, 8, 7), 12.0, (100.0, 90.0, 80.0))
    yield "random", rng.uniform(0, 300, (700, 3))
    yield "planar", synth.grid_points((20, 15, 1), 5.0, (50.0, 50.0, 30.0))
    yield "small", rng.uniform(0, 10, (20, 3))
    yield "clustered", np.concatenate([rng.normal(c, 2.0, (150, 3)) for c in ((20, 20, 20), (200, 40, 90))])


@pytest.mark.gpu
@pytest.mark.parametrize("name,pts", list(clouds()), ids=[c[0] for c in clouds()])
def test_gpu_order_neighbours_exact(name, pts):
    from digitalvolumecorrelation_gb300 import engine
    order, neigh = engine.order_neighbours(pts, k=75)
    o_ref, n_ref = reference_rule(pts, pts[0], 75)
    np.testing.assert_array_equal(order, o_ref)
    np.testing.assert_array_equal(neigh, n_ref)


@pytest.mark.gpu
def test_gpu_neighbours_match_host_up_to_ties(oracle):
    """Same neighbour distances as the reference-order host path; only the
    order among equal distances may differ."""
    from digitalvolumecorrelation_gb300 import engine, synth
    pts = synth.grid_points((8, 8, 8), 10.0, (50.0, 50.0, 50.0))
    order, neigh = engine.order_neighbours(pts, k=75)
    o_host, n_host = oracle.order_neighbours(pts)
    d = lambda i, j: np.sqrt(((pts[i] - pts[j]) ** 2).sum(-1))
    for i in range(len(pts)):
        np.testing.assert_array_equal(d(i, neigh[i]), d(i, n_host[i]))
    np.testing.assert_array_equal(d(0, order), d(0, o_host))
