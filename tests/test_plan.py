"""Several search configurations in one launch (dvc_gpu_plan_*), through the C
ABI, against the one-configuration engine and the FP64 oracle.

  * With caller seeds every point's result (status, objmin, all 12
    parameters, Gauss-Newton iterations) is bit-identical to the result its
    own configuration's engine gives at the same cluster width.
  * With the reference's neighbour seeding across configurations, each
    point's result matches the oracle run with the seed that point saw (the
    mean of its good neighbours processed before it, else rigid_trans):
    status identical, u, v, w within 1e-3 voxel, objmin within 1e-5 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (96, 96, 96)
CONFIGS = (
    dict(subvol_geom="cube", subvol_size=15, subvol_npts=600, obj_function="znssd", num_srch_dof=6,
         disp_max=4, basin_radius=2.0),
    dict(subvol_geom="sphere", subvol_size=17, subvol_npts=900, obj_function="ssd", num_srch_dof=12,
         disp_max=4, basin_radius=2.0),
    dict(subvol_geom="cube", subvol_size=13, subvol_npts=400, obj_function="znssd", num_srch_dof=3,
         disp_max=3, basin_radius=0.0),
    dict(subvol_geom="sphere", subvol_size=21, subvol_npts=1500, obj_function="znssd", num_srch_dof=6,
         disp_max=4, basin_radius=0.0),
)


@pytest.fixture(scope="module")
def case(gpu_lib):
    from digitalvolumecorrelation_gb300 import synth
    field = synth.Piecewise(t1=(1.0, -0.5, 0.5), E1=synth.rotation_z(1.5), c1=(24.0, 48.0, 48.0),
                            E2=((0, 0, 0), (0, 0, 0), (0, 0, -0.01)), c2=(48.0, 48.0, 48.0), split=48.0)
    blobs = synth.blobs(SHAPE, 900, seed=41)
    ref = synth.render(SHAPE, blobs, noise_sigma=2.0, noise_seed=42)
    cor = synth.render(SHAPE, blobs, deform=field, noise_sigma=2.0, noise_seed=43)
    rng = np.random.default_rng(44)
    pts = rng.uniform(22.0, 74.0, (160, 3))
    pts[0] = (24.0, 48.0, 48.0)
    cfg = rng.integers(0, len(CONFIGS), len(pts)).astype(np.int32)
    seeds = field.u(pts) + rng.normal(0.0, 0.6, pts.shape)
    return dict(ref=ref, cor=cor, pts=pts, cfg=cfg, seeds=seeds, field=field)


def _engines(case):
    from digitalvolumecorrelation_gb300 import engine
    from digitalvolumecorrelation_gb300.abi import make_params
    import torch
    pad = 64
    ref_d = torch.zeros(case["ref"].size + pad, dtype=torch.uint8, device="cuda")
    cor_d = torch.zeros(case["cor"].size + pad, dtype=torch.uint8, device="cuda")
    ref_d[: case["ref"].size] = torch.from_numpy(case["ref"].ravel())
    cor_d[: case["cor"].size] = torch.from_numpy(case["cor"].ravel())
    engines = [engine.Engine(make_params(SHAPE, interp_type="tricubic", **kw), ref_dev=ref_d, cor_dev=cor_d)
               for kw in CONFIGS]
    return engines, (ref_d, cor_d)


def _same(a, b):
    for k in ("status", "objmin", "params", "gn_iters"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("cluster", [2, 8])
def test_plan_matches_one_configuration_engines(case, cluster):
    from digitalvolumecorrelation_gb300 import engine
    engines, keep = _engines(case)
    plan = engine.Plan(engines, cluster=cluster)
    assert plan.info()["cluster"] == cluster
    r = plan.process(case["cfg"], case["pts"], seed_mode=engine.SEED_GIVEN, seeds=case["seeds"])
    assert (r["status"] == 0).mean() > 0.8
    for i, E in enumerate(engines):
        sel = np.nonzero(case["cfg"] == i)[0]
        E.set_cluster(cluster)
        s = E.process(case["pts"][sel], seed_mode=engine.SEED_GIVEN, seeds=case["seeds"][sel])
        _same({k: r[k][sel] for k in ("status", "objmin", "params", "gn_iters")}, s)
    plan.close()
    for E in engines:
        E.close()


def _seeds_seen(order, neigh, status, params, rigid):
    """The start translation each point saw under the reference's seeding:
    mean of its good neighbours processed before it, else rigid_trans
    (Core/Search.cpp:277-377)."""
    n = len(status)
    done = np.zeros(n, bool)
    seeds = np.zeros((n, 3))
    for m in order:
        nb = [j for j in neigh[m] if done[j] and status[j] == 0]
        seeds[m] = params[nb, :3].mean(0) if nb else rigid
        done[m] = True
    return seeds


def test_plan_neighbour_seeding_vs_oracle(case, oracle):
    from digitalvolumecorrelation_gb300 import engine, workloads
    from digitalvolumecorrelation_gb300.abi import make_params
    engines, keep = _engines(case)
    plan = engine.Plan(engines)
    order, neigh = workloads.order_and_neighbours(case["pts"])
    r = plan.process(case["cfg"], case["pts"], order=order, neigh=neigh)
    seeds = _seeds_seen(order, neigh, r["status"], r["params"], np.zeros(3))
    assert np.abs(seeds - case["field"].u(case["pts"])).max() < 1.5
    for i, kw in enumerate(CONFIGS):
        sel = np.nonzero(case["cfg"] == i)[0]
        p = make_params(SHAPE, interp_type="tricubic", **kw)
        o = oracle.process(p, case["ref"], case["cor"], case["pts"][sel], seed_mode=1, seeds=seeds[sel])
        np.testing.assert_array_equal(r["status"][sel], o["status"])
        good = o["status"] == 0
        assert good.mean() > 0.7
        assert np.abs(r["params"][sel][good, :3] - o["params"][good, :3]).max() <= 1e-3
        rel = np.abs(r["objmin"][sel][good] - o["objmin"][good]) / np.abs(o["objmin"][good])
        assert rel.max() <= 1e-5
    plan.close()
    for E in engines:
        E.close()


def test_plan_rejects_bad_configuration_index(case):
    from digitalvolumecorrelation_gb300 import engine
    engines, keep = _engines(case)
    plan = engine.Plan(engines)
    bad = case["cfg"].copy()
    bad[5] = len(CONFIGS)
    with pytest.raises(engine.DvcError) as ex:
        plan.process(bad, case["pts"], seed_mode=engine.SEED_GIVEN, seeds=case["seeds"])
    assert ex.value.code == engine.E_ARG
    plan.close()
    for E in engines:
        E.close()


def test_plan_rejects_engines_on_other_volumes(case):
    from digitalvolumecorrelation_gb300 import engine
    engines, keep = _engines(case)
    other, keep2 = _engines(case)
    with pytest.raises(engine.DvcError):
        engine.Plan([engines[0], other[1]])
    for E in engines + other:
        E.close()


def test_plan_autotune(case):
    """The autotuner times every launch shape that fits and keeps the fastest;
    results afterwards equal the one-configuration engines at that width."""
    import torch
    from digitalvolumecorrelation_gb300 import engine
    engines, keep = _engines(case)
    plan = engine.Plan(engines)
    n = len(case["pts"])
    dev = torch.device("cuda")
    t = lambda a, dt=None: torch.as_tensor(a, dtype=dt, device=dev)
    st = torch.empty(n, dtype=torch.int32, device=dev)
    ob = torch.empty(n, dtype=torch.float64, device=dev)
    pa = torch.empty((n, 12), dtype=torch.float64, device=dev)
    args = (t(case["cfg"]), n, t(case["pts"]), t(np.arange(n), torch.int32), n, None, 0,
            engine.SEED_GIVEN, t(case["seeds"]), st, ob, pa)
    times = plan.autotune(*args, reps=1)
    assert len(times) >= 4 and all(v > 0 for v in times.values())
    info = plan.info()
    best = min(times, key=times.get)
    assert (info["cluster"], info["staging"]) == best
    r = plan.process(case["cfg"], case["pts"], seed_mode=engine.SEED_GIVEN, seeds=case["seeds"])
    for i, E in enumerate(engines):
        sel = np.nonzero(case["cfg"] == i)[0]
        E.set_cluster(info["cluster"])
        s = E.process(case["pts"][sel], seed_mode=engine.SEED_GIVEN, seeds=case["seeds"][sel])
        _same({k: r[k][sel] for k in ("status", "objmin", "params", "gn_iters")}, s)
    plan.close()
    for E in engines:
        E.close()


def test_plan_launch_in_a_cuda_graph(case):
    """After one call has sized the workspace, the plan's launch (memsets,
    dataflow kernels, search) is captured in a CUDA graph; replays give
    exactly the results of the direct call (reference seeding across the
    configurations)."""
    import torch
    from digitalvolumecorrelation_gb300 import engine, workloads
    engines, keep = _engines(case)
    plan = engine.Plan(engines)
    n = len(case["pts"])
    order, neigh = workloads.order_and_neighbours(case["pts"])
    dev = torch.device("cuda")
    t = lambda a, dt=None: torch.as_tensor(a, dtype=dt, device=dev)
    cfg_d, pts_d, od, nd = t(case["cfg"]), t(case["pts"]), t(order), t(neigh)
    st = torch.empty(n, dtype=torch.int32, device=dev)
    ob = torch.empty(n, dtype=torch.float64, device=dev)
    pa = torch.empty((n, 12), dtype=torch.float64, device=dev)
    its = torch.empty(n, dtype=torch.int32, device=dev)

    def call(stream):
        plan.process_device(cfg_d, n, pts_d, od, n, nd, neigh.shape[1], engine.SEED_NEIGHBOURS, None, st, ob,
                            pa, its, stream=stream)

    call(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    direct = [x.clone() for x in (st, ob, pa, its)]
    for x in (st, ob, pa, its):
        x.zero_()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.graph(g, stream=side, capture_error_mode="thread_local"):
        call(side.cuda_stream)
    for _ in range(2):
        g.replay()
        torch.cuda.synchronize()
        for a, b in zip((st, ob, pa, its), direct):
            assert torch.equal(a, b)
    assert (direct[0] == 0).float().mean().item() > 0.8
    del g
    plan.close()
    for E in engines:
        E.close()
