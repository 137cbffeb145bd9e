"""The allocation-free search entry point, dvc_gpu_process_device_noalloc.

Some callers cannot allocate device memory at the moment they search: a host
program whose own pool owns all device memory, or one that records its work
while allocation is not allowed. They call the no-allocation variant, whose
scratch is a fixed array inside the library. This test calls it through the
C ABI twice in a row and checks each result against the ordinary
(allocating) entry point on the same inputs: identical status codes, and
parameters and objective within the tolerances of the other parity tests
(here far tighter, since both run the same kernel), and that the device's
free memory is the same before and after the calls. It also checks that a
point count above the array's capacity is refused.

The file name makes pytest collect it last, so a run that stops at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from fixtures import case_params, hotpath, search_cases

pytestmark = pytest.mark.gpu


def _bind(L):
    fn = L.dvc_gpu_process_device_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                   C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


@pytest.mark.parametrize("k", [1, 6, 0])
def test_noalloc_matches_allocating_entry_point(gpu_lib, k):
    import torch

    from digitalvolumecorrelation_gb300 import engine

    L = engine.load()
    noalloc = _bind(L)
    d = hotpath()
    case = search_cases()[k]
    vs = case["volumes"]
    E = engine.Engine(case_params(case), d[f"vol_{vs}_ref"], d[f"vol_{vs}_cor"])
    dev = torch.device("cuda")
    pts = torch.from_numpy(np.ascontiguousarray(d["search_points"])).to(dev)
    order = torch.from_numpy(np.ascontiguousarray(d["search_order"], np.int32)).to(dev)
    neigh = torch.from_numpy(np.ascontiguousarray(d["search_neigh"], np.int32)).to(dev)
    n, nn = len(d["search_points"]), d["search_neigh"].shape[1]

    def outputs():
        return (torch.empty(n, dtype=torch.int32, device=dev),
                torch.empty(n, dtype=torch.float64, device=dev),
                torch.empty((n, 12), dtype=torch.float64, device=dev),
                torch.empty(n, dtype=torch.int32, device=dev))

    st0, ob0, pa0, it0 = outputs()
    E.process_device(n, pts, order, n, neigh, nn, 0, None, st0, ob0, pa0, it0)
    torch.cuda.synchronize()
    ptr = lambda t: C.c_void_p(t.data_ptr())
    outs = [outputs(), outputs()]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for st, ob, pa, it in outs:  # two calls in a row share the library's scratch array
        rc = noalloc(E._h, n, ptr(pts), n, ptr(order), nn, ptr(neigh), 0, None, ptr(st), ptr(ob),
                     ptr(pa), ptr(it), None)
        assert rc == 0, L.dvc_gpu_last_error()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(st.cpu().numpy(), st0.cpu().numpy())
        np.testing.assert_allclose(pa.cpu().numpy(), pa0.cpu().numpy(), rtol=0, atol=1e-9)
        np.testing.assert_allclose(ob.cpu().numpy(), ob0.cpu().numpy(), rtol=1e-9, atol=0)
        np.testing.assert_array_equal(it.cpu().numpy(), it0.cpu().numpy())
        # and the reference's recorded answer
        np.testing.assert_array_equal(st.cpu().numpy(), d[f"search_{k}_status"])
        # the calls took no device memory: the device's free bytes are unchanged
        assert torch.cuda.mem_get_info()[0] == free0
    E.close()


def test_noalloc_rejects_more_points_than_its_capacity(gpu_lib):
    from digitalvolumecorrelation_gb300 import engine

    L = engine.load()
    noalloc = _bind(L)
    d = hotpath()
    E = engine.Engine(case_params(search_cases()[0]), d["vol_A_ref"], d["vol_A_cor"])
    rc = noalloc(E._h, 65536 + 1, None, 0, None, 0, None, 2, None, None, None, None, None, None)
    assert rc == -10
    assert b"DVC_NOALLOC_MAX_POINTS" in L.dvc_gpu_last_error()
    E.close()
