"""Device-side failures reach the caller, and the GPU stays usable.

The reference surfaces every failure of a point as an exception turned into a
status (Core/Utility.h:76-86, Core/dvc.cpp:233-303). The GPU search cannot
throw: every wait inside it (a point waiting for the neighbours the reference
processes first, a cluster waiting for a ready-queue slot, a staging copy
waiting on its barrier) is bounded, and a wait that gives up records
DVC_E_TIMEOUT in the launch's error flag. These tests make the dependency
waits run out on purpose, by a host-set limit of zero polls (no fault, no
trap, nothing left spinning), and check that:
  * the host-array call returns DVC_E_TIMEOUT;
  * device-array callers read it with dvc_gpu_last_status, for the
    dataflow-scheduled path, the in-order path and the allocation-free path;
  * the points whose wait gave up are left DVC_NOT_SEARCH;
  * the call returns promptly, and the next call with the default limit
    gives the reference's recorded answers.
"""
import ctypes as C
import time

import numpy as np
import pytest

from fixtures import case_params, hotpath, search_cases

pytestmark = pytest.mark.gpu

E_TIMEOUT = -13
NOT_SEARCH = -3


def _engine(k):
    from digitalvolumecorrelation_gb300 import engine
    d = hotpath()
    case = search_cases()[k]
    vs = case["volumes"]
    return d, engine.Engine(case_params(case), d[f"vol_{vs}_ref"], d[f"vol_{vs}_cor"])


def _check_reference_answer(d, k, r):
    np.testing.assert_array_equal(r["status"], d[f"search_{k}_status"])
    good = r["status"] == 0
    assert np.abs(r["params"][good, :3] - d[f"search_{k}_params"][good, :3]).max() <= 1e-3


def test_host_call_reports_a_dependency_wait_that_gave_up(gpu_lib):
    from digitalvolumecorrelation_gb300 import engine
    k = 0
    d, E = _engine(k)
    E.set_wait_limit(0)
    t0 = time.perf_counter()
    with pytest.raises(engine.DvcError) as ex:
        E.process(d["search_points"], order=d["search_order"], neigh=d["search_neigh"])
    assert ex.value.code == E_TIMEOUT
    assert time.perf_counter() - t0 < 20.0
    assert E.last_status() == E_TIMEOUT
    # the default limit again: the same engine gives the reference's answers
    E.set_wait_limit(-1)
    r = E.process(d["search_points"], order=d["search_order"], neigh=d["search_neigh"])
    _check_reference_answer(d, k, r)
    assert E.last_status() == 0
    E.close()


@pytest.mark.parametrize("in_order", [False, True])
def test_device_call_status_after_a_wait_gave_up(gpu_lib, monkeypatch, in_order):
    """dvc_gpu_process_device returns once enqueued; the timeout is read back
    with dvc_gpu_last_status. in_order: points in processing order, each
    waiting for its predecessors' flags (instead of the ready queue)."""
    import torch
    if in_order:
        monkeypatch.setenv("DVC_IN_ORDER", "1")
    k = 6
    d, E = _engine(k)
    dev = torch.device("cuda")
    pts = torch.from_numpy(np.ascontiguousarray(d["search_points"])).to(dev)
    order = torch.from_numpy(np.ascontiguousarray(d["search_order"], np.int32)).to(dev)
    neigh = torch.from_numpy(np.ascontiguousarray(d["search_neigh"], np.int32)).to(dev)
    n, nn = len(d["search_points"]), d["search_neigh"].shape[1]
    st = torch.empty(n, dtype=torch.int32, device=dev)
    ob = torch.empty(n, dtype=torch.float64, device=dev)
    pa = torch.empty((n, 12), dtype=torch.float64, device=dev)
    E.set_wait_limit(0)
    t0 = time.perf_counter()
    E.process_device(n, pts, order, n, neigh, nn, 0, None, st, ob, pa)
    assert E.last_status() == E_TIMEOUT
    assert time.perf_counter() - t0 < 20.0
    s = st.cpu().numpy()
    assert (s == NOT_SEARCH).sum() >= 1
    assert set(np.unique(s)) <= {0, -1, NOT_SEARCH}
    E.set_wait_limit(-1)
    E.process_device(n, pts, order, n, neigh, nn, 0, None, st, ob, pa)
    assert E.last_status() == 0
    r = dict(status=st.cpu().numpy(), params=pa.cpu().numpy())
    _check_reference_answer(d, k, r)
    E.close()


def test_allocation_free_call_status_after_a_wait_gave_up(gpu_lib):
    """The allocation-free search keeps its control block at a fixed place of
    its scratch array, so dvc_gpu_last_status reads its outcome too."""
    import torch

    from digitalvolumecorrelation_gb300 import engine
    L = engine.load()
    fn = L.dvc_gpu_process_device_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                   C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    k = 1
    d, E = _engine(k)
    dev = torch.device("cuda")
    pts = torch.from_numpy(np.ascontiguousarray(d["search_points"])).to(dev)
    order = torch.from_numpy(np.ascontiguousarray(d["search_order"], np.int32)).to(dev)
    neigh = torch.from_numpy(np.ascontiguousarray(d["search_neigh"], np.int32)).to(dev)
    n, nn = len(d["search_points"]), d["search_neigh"].shape[1]
    st = torch.empty(n, dtype=torch.int32, device=dev)
    ob = torch.empty(n, dtype=torch.float64, device=dev)
    pa = torch.empty((n, 12), dtype=torch.float64, device=dev)
    ptr = lambda t: C.c_void_p(t.data_ptr())
    for limit, expect in ((0, E_TIMEOUT), (-1, 0)):
        E.set_wait_limit(limit)
        rc = fn(E._h, n, ptr(pts), n, ptr(order), nn, ptr(neigh), 0, None, ptr(st), ptr(ob), ptr(pa),
                None, None)
        assert rc == 0, L.dvc_gpu_last_error()
        assert E.last_status() == expect
    _check_reference_answer(d, k, dict(status=st.cpu().numpy(), params=pa.cpu().numpy()))
    E.close()


def test_wait_limit_argument_checks(gpu_lib):
    from digitalvolumecorrelation_gb300 import engine
    L = engine.load()
    assert L.dvc_gpu_set_wait_limit(None, 5) == -10
    assert L.dvc_gpu_last_status(None) == -10
