"""DVC hot-path benchmark: ROI points/s of the GPU search on the
precision + scale configuration (1024^3 uint16 pair, 60,800-point grid,
sphere subvolumes of diameter 41 with 4000 samples, znssd, tricubic,
12 degrees of freedom), with the reference's own seeding semantics
(each point starts from its already-processed neighbours, in the
reference's processing order).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config 1|2]

A step is one full pass of the search over every ROI point. `value` is
points/s with volumes and point arrays resident in HBM (CUDA events on the
launch stream); `e2e` is the same through the C ABI with host buffers
(volume upload, search, result download inside the timed region). One JSON
line is printed by rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ROI points/s at <=0.01-voxel error vs FP64 oracle (plain GPU method)"

# FP32 work of one sample-evaluation as the search kernel performs it (the
# separable tricubic form): 64 stencil products + 16 + 4 for the y and z
# passes, 3 x 8 for the Catmull-Rom weights, ~8 for the warp and the
# compensated objective sums: about 100 FMA = 200 FLOP
FP32_FLOP_PER_SAMPLE = 200.0
FP32_LANES_PER_SM = 128


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=2, choices=[1, 2])
    ap.add_argument("--cpu-sample", type=int, default=384,
                    help="points of the workload timed on the CPU (cpu_baseline leg)")
    ap.add_argument("--ref-sample", type=int, default=64,
                    help="points per step of the reference arm (--impl reference): the first "
                         "points of the processing order")
    ap.add_argument("--profile-cnn", action="store_true",
                    help="one network forward pass over 1024 random patches, for profilers")
    ap.add_argument("--profile-learned", action="store_true",
                    help="the profile case in the learned search's form (12 start parameters, no grid)")
    ap.add_argument("--profile-case", action="store_true",
                    help="one search launch on a small case for profilers: the bench "
                         "configuration's subvolumes and search on 384^3 uint16 volumes, "
                         "216 points with given seeds")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned-initial-guess comparison (configuration 4)")
    ap.add_argument("--learned-steps", type=int, default=3000)
    ap.add_argument("--no-batching", action="store_true",
                    help="skip configuration 3 (60 configurations in one launch)")
    ap.add_argument("--no-pipeline", action="store_true",
                    help="skip configuration 5 (8 GiB pair, 499,200 points, learned + plain; needs "
                         "the learned leg's network)")
    ap.add_argument("--pipeline-only", action="store_true",
                    help="train the network (learned leg) and run only configuration 5")
    ap.add_argument("--batching-only", action="store_true",
                    help="run only the configuration 3 leg and print its JSON")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(ms, world, device=None):
    """The slowest rank's step time: all-reduce MAX of `ms` over the process
    group (replicas: each rank searches its own copy of the workload)."""
    if world <= 1:
        return float(ms)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(n_points, world, ms):
    """Whole-job points/s: every rank's points over the slowest rank's time."""
    return n_points * world / (ms / 1e3)


def workload(cfg):
    from digitalvolumecorrelation_gb300 import workloads
    return workloads.config1() if cfg == 1 else workloads.config2()


def bench_config(W, world):
    """The `config` object of both arms' JSON lines (the same workload)."""
    from digitalvolumecorrelation_gb300.synth import cube_subvol_count
    p = W.params()
    n_sub = p.subvol_npts if p.subvol_geom == 1 else cube_subvol_count(p.subvol_npts)
    return {"workload": W.name, "points": len(W.points), "volume": list(W.shape),
            "bytes_per_voxel": W.bytes_per_voxel, "n_sub": n_sub,
            "seeding": "reference (neighbours, processing order)",
            "l2": "inputs larger than L2 (two %d MiB volumes)" % (W.nvox * W.bytes_per_voxel >> 20),
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "params": W.params_kw}


class Clocks:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        # raw samples: DVC_CLOCKS_DIR (default: the system temporary directory)
        out_dir = os.environ.get("DVC_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out_dir, f"dvc_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def seeds_from_results(order, neigh, status, params, rigid, n_process):
    """The reference's start estimate for each point (Core/Search.cpp:277-377)
    recomputed on the host from the finished results."""
    n = len(status)
    rank = np.full(n, np.iinfo(np.int32).max, np.int64)
    rank[order[:n_process]] = np.arange(n_process)
    seeds = np.tile(np.asarray(rigid, np.float64), (n, 1))
    for i in order[:n_process]:
        nb = neigh[i]
        ok = (rank[nb] < rank[i]) & (status[nb] == 0)
        if ok.any():
            seeds[i] = params[nb[ok], :3].sum(0) / ok.sum()
    return seeds


def cpu_leg(W, p, ref_np, cor_np, pts, seeds, gpu, sample, threads):
    """The FP64 oracle (a port of the reference path) on a bounded sample of
    points with the GPU run's seeds: its time, and the GPU's agreement with
    it on the metric's terms (status, u/v/w, objmin)."""
    from oracle.oracle import Oracle
    O = Oracle()
    idx = sample
    t0 = time.perf_counter()
    r = O.process(p, ref_np, cor_np, pts[idx], seed_mode=1, seeds=seeds[idx], n_threads=threads)
    dt = time.perf_counter() - t0
    st, ob, pa = gpu["status"][idx], gpu["objmin"][idx], gpu["params"][idx]
    good = (r["status"] == 0) & (st == 0)
    acc = {"same_status": int((r["status"] == st).sum()), "points": len(idx),
           "max_abs_du_gpu_vs_oracle_vox": float(np.abs(r["params"][good, :3] - pa[good, :3]).max())
           if good.any() else None,
           "max_rel_objmin_gpu_vs_oracle": float((np.abs(ob[good] - r["objmin"][good]) /
                                                  np.abs(r["objmin"][good])).max()) if good.any() else None}
    return len(idx) / dt, dt, acc, r


def profile_case(learned=False):
    """One launch of the search kernel on a case small enough for ncu's
    replays: the bench configuration's sphere subvolumes (41 voxels, 4000
    samples), znssd, tricubic, 12 degrees of freedom, disp_max 6 / basin 3, on
    384^3 uint16 volumes (2 x 113 MB, more than L2), 216 points, seeds within
    half a voxel of the truth. learned: the learned search's form instead,
    1728 points started from all 12 parameters (translations within 0.7
    voxel RMS of the truth, rotations and strains of the network's error
    size), no coarse grid: the kernel built for two CTAs per SM."""
    import torch
    from digitalvolumecorrelation_gb300 import engine, synth, workloads
    shape = (384, 384, 384)
    pts = (synth.grid_points((12, 12, 12), 12.0, (192.0, 192.0, 192.0)) if learned
           else synth.grid_points((6, 6, 6), 24.0, (192.0, 192.0, 192.0)))
    kw = dict(subvol_geom="sphere", subvol_size=41, subvol_npts=4000, obj_function="znssd",
              interp_type="tricubic", num_srch_dof=12, disp_max=6, basin_radius=3.0)
    b = synth.blobs(shape, int(np.prod(shape) // 1000), sigma=(1.5, 3.0), amp=(2000.0, 60000.0), seed=2)
    W = workloads.Workload("profile_384cube_u16_216pts_sphere41_dof12", shape, 2, kw, pts,
                           synth.Sinusoid(A=3.0, L=400.0), b, 150.0, 201, 202)
    p = W.params()
    n = len(pts)
    ref_d, cor_d = W.render_device()
    E = engine.Engine(p, ref_dev=ref_d, cor_dev=cor_d)
    dev = torch.device("cuda")
    rng = np.random.default_rng(0)
    if learned:
        seeds = np.zeros((n, 12))
        seeds[:, :3] = W.truth() + rng.normal(0, 0.7, (n, 3))
        seeds[:, 3:6] = rng.normal(0, 0.004, (n, 3))
        seeds[:, 6:] = rng.normal(0, 0.006, (n, 6))
    else:
        seeds = W.truth() + rng.normal(0, 0.5, (n, 3))
    t = lambda a, dt=None: torch.as_tensor(a, dtype=dt, device=dev)
    st = torch.empty(n, dtype=torch.int32, device=dev)
    ob = torch.empty(n, dtype=torch.float64, device=dev)
    pa = torch.empty((n, 12), dtype=torch.float64, device=dev)
    it = torch.empty(n, dtype=torch.int32, device=dev)
    mode = engine.SEED_PARAMS if learned else engine.SEED_GIVEN
    E.process_device(n, t(W.points), t(np.arange(n), torch.int32), n, None, 0, mode, t(seeds), st, ob,
                     pa, it, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": W.name + ("_learned_start" if learned else ""),
                      "good": int((st == 0).sum().item()), "points": n, "launch": E.last_launch(),
                      "evaluations": E.last_counters()[0], "sample_evals": E.last_counters()[0] * 4000}))


def profile_cnn(batch=1024, passes=3):
    """The learned proposer's forward pass (patches to 12 parameters) over a
    batch of 1024 random patches, `passes` times (random weights: the cost
    does not depend on them)."""
    import torch
    from digitalvolumecorrelation_gb300 import engine
    net = engine.Cnn(seed=3)
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.randn((batch, 2, 32, 32, 32), generator=g, device="cuda", dtype=torch.float32)
    y = torch.empty((batch, 12), dtype=torch.float32, device="cuda")
    for _ in range(passes):
        net.forward(batch, x, y)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    net.forward(batch, x, y)
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    # algorithmic FLOPs per patch: the four convolutions (2 Cout Cin 27 per
    # output voxel) and the two dense layers
    conv = sum(2 * co * ci * 27 * (d // 2) ** 3 for ci, co, d in ((2, 16, 32), (16, 32, 16), (32, 64, 8), (64, 96, 4)))
    flop = batch * (conv + 2 * 768 * 128 + 2 * 128 * 12)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("bf16_tflops", 1900.0)
    tf = flop / (ms / 1e3) / 1e12
    print(json.dumps({"profile_cnn": batch, "forward_ms": round(ms, 3), "patches_per_s": round(batch / ms * 1e3),
                      "gflop": round(flop / 1e9, 2), "tflops": round(tf, 1), "frac_of_bf16_peak": round(tf / peak, 4),
                      "convolutions": "FP32 CUDA cores" if os.environ.get("DVC_CNN_FP32") else "tcgen05 BF16"}))
    net.close()


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.profile_case or args.profile_learned:
        return profile_case(learned=args.profile_learned)
    if args.profile_cnn:
        return profile_cnn()
    if args.pipeline_only:
        import torch
        torch.cuda.set_device(local)
        summary, weights = learned_leg(args.learned_steps)
        print(json.dumps({"learned": summary, "pipeline": pipeline_leg(weights)}))
        return
    if args.batching_only:
        import torch
        torch.cuda.set_device(local)
        print(json.dumps({"batching": batching_leg()}))
        return

    import torch
    from digitalvolumecorrelation_gb300 import engine, workloads
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    W = workload(args.config)
    p = W.params()
    n = len(W.points)
    order, neigh = workloads.order_and_neighbours(W.points)
    ref_d, cor_d = W.render_device()
    E = engine.Engine(p, ref_dev=ref_d, cor_dev=cor_d)
    dev = torch.device("cuda", local)
    pts_d = torch.from_numpy(W.points).to(dev)
    order_d = torch.from_numpy(order).to(dev)
    neigh_d = torch.from_numpy(neigh).to(dev)
    status_d = torch.empty(n, dtype=torch.int32, device=dev)
    objmin_d = torch.empty(n, dtype=torch.float64, device=dev)
    params_d = torch.empty((n, 12), dtype=torch.float64, device=dev)
    its_d = torch.empty(n, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream

    def step():
        E.process_device(n, pts_d, order_d, n, neigh_d, neigh.shape[1], 0, None, status_d,
                         objmin_d, params_d, its_d, stream=stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = Clocks(local)
    clk.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        step()
    ev1.record()
    torch.cuda.synchronize()
    clocks = clk.stop()
    device_status = E.last_status()  # a bounded wait that gave up would show here
    if device_status != 0:
        raise SystemExit(f"search launch reported device status {device_status}")
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, world, dev)
    # the search's launches per step: one per non-empty rank window
    w1, w2, wide = E.last_windows()
    search_launches = sum(1 for lo, hi in ((0, w1), (w1, w2), (w2, n)) if hi > lo)
    launch = dict(E.last_launch(), windows={"first": w1, "last": n - w2, "cluster": wide})
    status = status_d.cpu().numpy()
    params = params_d.cpu().numpy()
    objmin = objmin_d.cpu().numpy()
    its = its_d.cpu().numpy()
    value = replica_value(n, world, ms)

    # sample-evaluations per launch (the roofline's unit), from the counts the
    # engine keeps: per point, the reference subvolume, every grid offset, each
    # Gauss-Newton evaluation and the final objective, times the samples
    from digitalvolumecorrelation_gb300.synth import cube_subvol_count
    n_sub = p.subvol_npts if p.subvol_geom == 1 else cube_subvol_count(p.subvol_npts)
    k = int(p.disp_max / p.basin_radius) if p.basin_radius else 0
    grid = (2 * k + 1) ** 3 if p.basin_radius else 0
    good = status == 0
    evals, gn_total, undefined = E.last_counters()  # of the last timed step
    ph = np.array(E.last_phase_cycles(), float)  # SM cycles per phase, all CTAs, last step
    phase_names = ("take_work_and_seed", "setup", "grid", "gn_entry_exit", "final", "gn_warp", "gn_range_stage",
                   "gn_eval", "gn_reduce", "gn_solve")
    phase_shares = {k: round(float(v / ph[:10].sum()), 4) for k, v in zip(phase_names, ph[:10])} if ph[:10].sum() else {}
    sample_evals = evals * n_sub
    flop_per_sample = 8192.0  # fused 64x64 stencil-coefficient product per sample-evaluation
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak_tf = peaks.get("bf16_tflops", 1900.0)
    achieved = sample_evals * flop_per_sample / (ms / 1e3) / 1e12
    # the FP32 pipes' peak at the clock seen in the timed region: every SM's
    # 128 FP32 lanes, one FMA (2 FLOP) per lane per cycle
    props = torch.cuda.get_device_properties(dev)
    sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    fp32_peak = props.multi_processor_count * FP32_LANES_PER_SM * 2.0 * sm_mhz * 1e6 / 1e12
    fp32_achieved = sample_evals * FP32_FLOP_PER_SAMPLE / (ms / 1e3) / 1e12

    # accuracy: truth and oracle sample
    truth = W.truth()
    err_truth = np.abs(params[good, :3] - truth[good]).max() if good.any() else None
    result = {
        "metric": METRIC, "value": round(value, 2), "unit": "points/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded speckle pair rendered on the GPU; no public dataset)",
        "config": bench_config(W, world),
        # per step: outputs initialised, ranks, and for the dataflow schedule the
        # dependency count, prefix sum, successor fill and ready queue; the
        # search (one launch per rank window)
        "gpu_launches": (6 + search_launches) * args.steps,
        "launch": launch,
        "device_status": device_status,
        "results": {"good": int(good.sum()), "range_fail": int((status == -1).sum()),
                    "mean_gn_iters": float(its[good].mean()) if good.any() else None,
                    "evaluations": evals, "undefined_cell_evaluations": undefined,
                    # share of the CTAs' SM cycles per phase of the point loop
                    # (gn_eval includes the G'G accumulation)
                    "phase_shares": phase_shares,
                    "max_abs_err_vs_truth_vox": None if err_truth is None else float(err_truth),
                    "median_abs_err_vs_truth_vox": float(np.median(np.abs(params[good, :3] - truth[good])))
                    if good.any() else None},
        "roofline": {"bound": "tensor", "achieved": round(achieved, 2), "peak": peak_tf,
                     "unit": "TFLOP/s", "frac": round(achieved / peak_tf, 4),
                     "traffic": None,
                     "traffic_note": "DRAM bytes are not measurable inside the run; a one-pass ncu "
                                     "capture of the search (one launch, before the rank windows) "
                                     "read 2.1x the algorithmic bytes",
                     "flop_per_unit": flop_per_sample, "units_per_launch": sample_evals,
                     "peak_source": "measured bf16 (burst)" if "bf16_tflops" in peaks else "fallback",
                     "note": "algorithmic FLOPs of the fused 64x64 coefficient product per "
                             "sample-evaluation; the kernel evaluates the same interpolant in "
                             "separable form on the FP32 pipes (roofline_fp32)"},
        "roofline_fp32": {"bound": "fp32", "achieved": round(fp32_achieved, 2), "peak": round(fp32_peak, 1),
                          "unit": "TFLOP/s", "frac": round(fp32_achieved / fp32_peak, 4),
                          "flop_per_unit": FP32_FLOP_PER_SAMPLE, "units_per_launch": sample_evals,
                          "peak_source": f"{props.multi_processor_count} SMs x {FP32_LANES_PER_SM} FP32 "
                                         f"lanes x 2 FLOP x {sm_mhz:.0f} MHz (median SM clock of the run)",
                          "note": "the FP32 work the kernel performs per sample-evaluation; the rest of a "
                                  "point's time is its serial sections and the seeding's dependency chain"},
        "clocks": clocks,
    }
    if rank == 0 and not args.no_e2e:
        result["e2e"] = e2e_leg(W, p, order, neigh, ref_d, cor_d, n)
    if rank == 0 and not args.no_cpu and world == 1:
        seeds = seeds_from_results(order, neigh, status, params, p.rigid_trans[:], n)
        sample = order[:: max(1, n // args.cpu_sample)][: args.cpu_sample]
        ref_np = ref_d[: W.nvox].cpu().numpy()
        cor_np = cor_d[: W.nvox].cpu().numpy()
        if W.bytes_per_voxel == 2:
            ref_np = ref_np.view(np.uint16)
            cor_np = cor_np.view(np.uint16)
        threads = os.cpu_count() or 1
        gpu = dict(status=status, objmin=objmin, params=params)
        pps, dt, acc, _ = cpu_leg(W, p, ref_np, cor_np, W.points, seeds, gpu, sample, threads)
        result["cpu_baseline"] = {"value": round(pps, 4), "unit": "points/s", "cores": threads,
                                  "kind": "port", "seconds": round(dt, 2),
                                  "sample": f"{len(sample)} points of the same workload (evenly "
                                            "spaced in processing order) with the GPU run's seeds",
                                  "accuracy": acc}
    if rank == 0 and not args.no_learned and world == 1:
        result["learned"], weights = learned_leg(args.learned_steps)
        if not args.no_pipeline:
            result["pipeline"] = pipeline_leg(weights)
    if rank == 0 and not args.no_batching and world == 1:
        result["batching"] = batching_leg()
    if rank == 0:
        print(json.dumps(result))
    if world > 1:
        dist.destroy_process_group()


def learned_leg(steps, oracle_sample=32):
    """Configuration 4: the learned initial guess trained on the GPU, then the
    plain and the learned method on a held-out pair, both checked against the
    FP64 oracle on a sample of points (from the true translation, no grid:
    the converged optimum)."""
    from digitalvolumecorrelation_gb300 import learned
    from digitalvolumecorrelation_gb300.abi import make_params
    from oracle.oracle import Oracle
    summary, held, res, weights = learned.run(steps=steps, keep=True)
    rng = np.random.default_rng(5)
    n = len(held.points)
    sample = np.sort(rng.choice(n, oracle_sample, replace=False))
    shape = learned.SHAPE
    ref = held.ref[: held.w.nvox].cpu().numpy().reshape(shape[::-1])
    cor = held.cor[: held.w.nvox].cpu().numpy().reshape(shape[::-1])
    p0 = make_params(shape, **dict(learned.SEARCH, basin_radius=0.0))
    o = Oracle().process(p0, ref, cor, held.points[sample], seed_mode=1, seeds=held.truth[sample],
                         n_threads=os.cpu_count() or 1)
    ok = o["status"] == 0
    for name in ("plain", "plain_125", "learned"):
        st, pa = res[name]
        good = ok & (st[sample] == 0)
        err = np.abs(pa[sample][good, :3] - o["params"][good, :3]).max(axis=1)
        summary[name]["oracle_sample"] = int(ok.sum())
        summary[name]["within_0p01_vox_of_oracle"] = float(np.mean(err <= 0.01)) if len(err) else None
        summary[name]["max_err_vs_oracle_vox"] = float(err.max()) if len(err) else None
    return summary, weights


def pipeline_leg(weights, obj_threshold=0.1, oracle_sample=64, cpu_sample=512):
    """Configuration 5: the full pipeline on the 8 GiB uint16 pair and the
    499,200-point grid. The plain GPU method (reference seeding in processing
    order, coarse grid, Gauss-Newton) and the learned method (the network
    trained in the learned leg proposes all 12 parameters, Gauss-Newton
    refines, the plain search redoes points whose ZNSSD exceeds 0.1), each
    timed over one full pass after a warm-up pass; both checked against the
    FP64 oracle's converged optimum (started from the true translation, no
    grid) on a random sample; the reference's CPU path (the oracle with the
    plain run's seeds, full search) timed on a sample in processing order;
    neighbour lists from the GPU kNN and the strain window (5 points) fitted
    on the GPU."""
    import torch
    from digitalvolumecorrelation_gb300 import engine, workloads
    from digitalvolumecorrelation_gb300.abi import make_params
    from oracle.oracle import Oracle
    W = workloads.config5()
    n = len(W.points)
    t0 = time.perf_counter()
    ref_d, cor_d = W.render_device()
    render_s = time.perf_counter() - t0
    p = W.params()
    E = engine.Engine(p, ref_dev=ref_d, cor_dev=cor_d)
    t0 = time.perf_counter()
    order, neigh = engine.order_neighbours(W.points, k=75)
    knn_s = time.perf_counter() - t0
    net = engine.Cnn()
    net.set_weights(weights)
    dev = torch.device("cuda")
    pts_d, order_d, neigh_d = (torch.from_numpy(a).to(dev) for a in (W.points, order, neigh))
    truth = W.truth()
    out, res = {}, {}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for name in ("plain", "learned"):
        st = torch.empty(n, dtype=torch.int32, device=dev)
        ob = torch.empty(n, dtype=torch.float64, device=dev)
        pa = torch.empty((n, 12), dtype=torch.float64, device=dev)
        it = torch.empty(n, dtype=torch.int32, device=dev)
        if name == "plain":
            run = lambda: E.process_device(n, pts_d, order_d, n, neigh_d, neigh.shape[1], engine.SEED_NEIGHBOURS,
                                           None, st, ob, pa, it)
        else:
            run = lambda: E.process_learned(net, n, pts_d, order_d, n, obj_threshold, st, ob, pa, it)
        run()
        torch.cuda.synchronize()
        ev0.record()
        fb = run()
        ev1.record()
        torch.cuda.synchronize()
        secs = ev0.elapsed_time(ev1) / 1e3
        s_, o_, p_ = st.cpu().numpy(), ob.cpu().numpy(), pa.cpu().numpy()
        res[name] = (s_, o_, p_)
        good = s_ == 0
        out[name] = dict(points_per_s=round(n / secs, 1), seconds=round(secs, 3), good=int(good.sum()),
                         median_abs_err_vs_truth_vox=float(np.median(np.abs(p_[good, :3] - truth[good]))),
                         mean_gn_iterations=float(it.float().mean().item()))
        if name == "learned":
            out[name]["fallback_points"] = int(fb)
            out[name]["fallback_rate"] = round(fb / n, 4)
    out["speedup_learned_over_plain"] = round(out["learned"]["points_per_s"] / out["plain"]["points_per_s"], 2)
    net.close()
    E.close()
    nvox = W.nvox
    ref_np = ref_d[:nvox].cpu().numpy().view(np.uint16).reshape(W.shape[::-1])
    cor_np = cor_d[:nvox].cpu().numpy().view(np.uint16).reshape(W.shape[::-1])
    del ref_d, cor_d
    O = Oracle()
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(6)
    sample = np.sort(rng.choice(n, oracle_sample, replace=False))
    p0 = make_params(W.shape, bytes_per_voxel=2, **dict(W.params_kw, basin_radius=0.0))
    o = O.process(p0, ref_np, cor_np, W.points[sample], seed_mode=1, seeds=truth[sample], n_threads=threads)
    ok = o["status"] == 0
    for name in ("plain", "learned"):
        s_, _, p_ = res[name]
        good = ok & (s_[sample] == 0)
        err = np.abs(p_[sample][good, :3] - o["params"][good, :3]).max(axis=1)
        out[name]["oracle_sample"] = int(ok.sum())
        out[name]["within_0p01_vox_of_oracle"] = float(np.mean(err <= 0.01)) if len(err) else None
        out[name]["max_err_vs_oracle_vox"] = float(err.max()) if len(err) else None
    # the reference's CPU path on a sample in processing order, with the plain run's seeds
    s_, _, p_ = res["plain"]
    seeds = seeds_from_results(order, neigh, s_, p_, p.rigid_trans[:], n)
    sub = order[:: max(1, n // cpu_sample)][:cpu_sample]
    t0 = time.perf_counter()
    o2 = O.process(p, ref_np, cor_np, W.points[sub], seed_mode=1, seeds=seeds[sub], n_threads=threads)
    cpu_s = time.perf_counter() - t0
    g2 = (o2["status"] == 0) & (s_[sub] == 0)
    # strain window of 5 points on the learned run's results
    s_, o_, p_ = res["learned"]
    t0 = time.perf_counter()
    sw = engine.strain(W.points, s_, o_, p_[:, :3], neigh, ndp=5)
    strain_s = time.perf_counter() - t0
    out.update({
        "workload": W.name, "points": n, "obj_threshold": obj_threshold, "render_seconds": round(render_s, 2),
        "knn_seconds": round(knn_s, 3), "strain_window": 5, "strain_seconds": round(strain_s, 3),
        "strain_points_fitted": int((sw["pts_in_sw"] >= 5).sum()),
        "reference_cpu": {"points_per_s": round(len(sub) / cpu_s, 3), "seconds": round(cpu_s, 2),
                          "threads": threads, "sample": f"{len(sub)} points evenly spaced in processing order, "
                                                        "the plain run's seeds, full search",
                          "same_status_as_gpu": int((o2["status"] == res["plain"][0][sub]).sum()),
                          "max_abs_du_gpu_vs_oracle_vox": float(np.abs(o2["params"][g2, :3] -
                                                                       res["plain"][2][sub][g2, :3]).max())
                          if g2.any() else None},
    })
    out["plain"]["speedup_over_reference_cpu"] = round(out["plain"]["points_per_s"] / (len(sub) / cpu_s), 1)
    return out


BATCHING_ORACLE_CONFIGS = ((21, "cube", 3, "ssd"), (41, "sphere", 12, "znssd"), (61, "cube", 6, "znssd"),
                           (81, "sphere", 12, "ssd"))


def batching_leg(steps=2, warmup=1, tune_points=4000, oracle_per_config=16):
    """Configuration 3: 40,000 scattered points, each with its own search
    configuration (60 in all), searched by one persistent launch of a plan
    whose launch shape the autotuner picks; the launch is also captured in a
    CUDA graph and replayed. Neighbour order and lists from the GPU kNN, the
    strain window (7 points) fitted on the GPU afterwards. A sample of points
    of four configurations is checked against the FP64 oracle with the seeds
    those points saw."""
    import torch
    from digitalvolumecorrelation_gb300 import engine, workloads
    from digitalvolumecorrelation_gb300.abi import make_params
    W, cfg, settings = workloads.config3()
    n = len(W.points)
    ref_d, cor_d = W.render_device()
    engines = [engine.Engine(make_params(W.shape, bytes_per_voxel=1, **kw), ref_dev=ref_d, cor_dev=cor_d)
               for kw in settings]
    t0 = time.perf_counter()
    order, neigh = engine.order_neighbours(W.points, start=W.points[0], k=75)
    knn_s = time.perf_counter() - t0
    plan = engine.Plan(engines)
    shape0 = plan.info()
    dev = torch.device("cuda")
    t = lambda a, dt=None: torch.as_tensor(a, dtype=dt, device=dev)
    cfg_d, pts_d, order_d, neigh_d = t(cfg), t(W.points), t(order), t(neigh)
    st = torch.empty(n, dtype=torch.int32, device=dev)
    ob = torch.empty(n, dtype=torch.float64, device=dev)
    pa = torch.empty((n, 12), dtype=torch.float64, device=dev)
    its = torch.empty(n, dtype=torch.int32, device=dev)
    # autotune on the first points of the processing order
    tune = plan.autotune(cfg_d, n, pts_d, order_d, min(tune_points, n), neigh_d, neigh.shape[1],
                         engine.SEED_NEIGHBOURS, None, st, ob, pa, reps=1)
    stream = torch.cuda.current_stream()

    def step():
        plan.process_device(cfg_d, n, pts_d, order_d, n, neigh_d, neigh.shape[1], engine.SEED_NEIGHBOURS,
                            None, st, ob, pa, its, stream=stream.cuda_stream)

    for _ in range(max(1, warmup)):
        step()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(steps):
        step()
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    # the same launch captured once in a CUDA graph and replayed
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side, capture_error_mode="thread_local"):
            plan.process_device(cfg_d, n, pts_d, order_d, n, neigh_d, neigh.shape[1], engine.SEED_NEIGHBOURS,
                                None, st, ob, pa, its, stream=side.cuda_stream)
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    ev0.record()
    for _ in range(steps):
        g.replay()
    ev1.record()
    torch.cuda.synchronize()
    ms_graph = ev0.elapsed_time(ev1) / steps
    status, objmin, params = st.cpu().numpy(), ob.cpu().numpy(), pa.cpu().numpy()
    good = status == 0
    truth = W.truth()
    # strain window of 7 points over the scattered cloud
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sw = engine.strain(W.points, status, objmin, params[:, :3], neigh, ndp=7)
    strain_s = time.perf_counter() - t0
    # oracle sample
    from oracle.oracle import Oracle
    O = Oracle()
    seeds = seeds_from_results(order, neigh, status, params, (0.0, 0.0, 0.0), n)
    ref_np = ref_d[: W.nvox].cpu().numpy().reshape(W.shape[::-1])
    cor_np = cor_d[: W.nvox].cpu().numpy().reshape(W.shape[::-1])
    rank = np.empty(n, np.int64)
    rank[order] = np.arange(n)
    errs, same_status, checked, osec = [], 0, 0, 0.0
    threads = os.cpu_count() or 1
    for size, geom, dof, obj in BATCHING_ORACLE_CONFIGS:
        ci = [i for i, kw in enumerate(settings) if (kw["subvol_size"], kw["subvol_geom"], kw["num_srch_dof"],
                                                      kw["obj_function"]) == (size, geom, dof, obj)][0]
        members = np.nonzero(cfg == ci)[0]
        members = members[np.argsort(rank[members])]
        sel = members[:: max(1, len(members) // oracle_per_config)][:oracle_per_config]
        p = make_params(W.shape, bytes_per_voxel=1, **settings[ci])
        t1 = time.perf_counter()
        o = O.process(p, ref_np, cor_np, W.points[sel], seed_mode=1, seeds=seeds[sel], n_threads=threads)
        osec += time.perf_counter() - t1
        checked += len(sel)
        same_status += int((o["status"] == status[sel]).sum())
        ok = (o["status"] == 0) & (status[sel] == 0)
        if ok.any():
            errs.append(np.abs(o["params"][ok, :3] - params[sel][ok, :3]).max(axis=1))
    err = np.concatenate(errs) if errs else np.zeros(0)
    plan_shape = plan.info()
    plan.close()
    for E in engines:
        E.close()
    return {
        "workload": W.name, "points": n, "configurations": len(settings),
        "value": round(n / (ms / 1e3), 2), "unit": "points/s", "ms_per_step": round(ms, 2),
        "graph_replay": {"value": round(n / (ms_graph / 1e3), 2), "ms_per_step": round(ms_graph, 2)},
        "launch_shape": plan_shape, "default_shape": shape0,
        "autotune_ms": {f"C{c}_stage{s_}": round(v, 2) for (c, s_), v in tune.items()},
        "autotune_sample_points": min(tune_points, n),
        "seeding": "reference (neighbours, processing order; order and lists from the GPU kNN)",
        "knn_seconds": round(knn_s, 3), "strain_window": 7, "strain_seconds": round(strain_s, 3),
        "strain_points_fitted": int((sw["pts_in_sw"] >= 7).sum()),
        "good": int(good.sum()), "range_fail": int((status == -1).sum()),
        "convg_fail": int((status == -2).sum()),
        "median_abs_err_vs_truth_vox": float(np.median(np.abs(params[good, :3] - truth[good]))),
        "oracle_sample": checked, "oracle_same_status": same_status,
        "within_0p01_vox_of_oracle": float(np.mean(err <= 0.01)) if len(err) else None,
        "max_err_vs_oracle_vox": float(err.max()) if len(err) else None,
        "oracle_points_per_s": round(checked / osec, 3), "oracle_threads": threads,
    }


def e2e_leg(W, p, order, neigh, ref_d, cor_d, n, iters=3):
    """Through the C ABI with host buffers: upload both volumes from pinned
    host memory, search, read back all results."""
    import torch
    from digitalvolumecorrelation_gb300 import engine
    ref_h = ref_d[: W.nvox].cpu().pin_memory()
    cor_h = cor_d[: W.nvox].cpu().pin_memory()
    ref_np = ref_h.numpy()
    cor_np = cor_h.numpy()
    if W.bytes_per_voxel == 2:
        ref_np = ref_np.view(np.uint16)
        cor_np = cor_np.view(np.uint16)
    times, parts = [], []
    for it in range(1 + iters):  # one untimed warm-up call, then `iters` timed ones
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        E = engine.Engine(p, ref_np, cor_np)
        t1 = time.perf_counter()
        r = E.process(W.points, order=order, neigh=neigh)
        t2 = time.perf_counter()
        E.close()
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        times.append(t3 - t0)
        parts.append((t1 - t0, t2 - t1, t3 - t2))
    dt = statistics.median(times[1:])
    h2d = 2 * W.nvox * W.bytes_per_voxel + W.points.nbytes + order.nbytes + neigh.nbytes
    d2h = n * (4 + 8 + 96 + 4)
    return {"value": round(n / dt, 2), "unit": "points/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "seconds": round(dt, 3),
            "timing": f"median of {iters} calls after one warm-up call",
            "seconds_each": [round(t, 3) for t in times[1:]],
            # per call: engine creation (both volumes uploaded), the search
            # call (arrays in, search, results out), engine destruction
            "seconds_create_search_destroy": [[round(v, 3) for v in q] for q in parts[1:]]}


def run_reference(args, rank, world):
    """The reference's CPU implementation of the path on the host cores, on
    the GPU arm's workload: the FP64 port of its search (oracle/; the
    reference's own sources are not on this machine to build), with the
    reference's seeding over the first --ref-sample points of the same
    processing order (the reference's own `num_points_to_process` subset),
    on the same two volumes, rendered by the same generator outside the
    timed region and copied to host memory. Every step searches that prefix
    again; all host threads."""
    if rank != 0:
        return
    import torch
    from digitalvolumecorrelation_gb300 import workloads
    from oracle.oracle import Oracle
    W = workload(args.config)
    p = W.params()
    order, neigh = workloads.order_and_neighbours(W.points)
    ref_d, cor_d = W.render_device()
    ref_np = ref_d[: W.nvox].cpu().numpy()
    cor_np = cor_d[: W.nvox].cpu().numpy()
    del ref_d, cor_d
    torch.cuda.empty_cache()
    if W.bytes_per_voxel == 2:
        ref_np, cor_np = ref_np.view(np.uint16), cor_np.view(np.uint16)
    n_sample = max(1, min(args.ref_sample, len(W.points)))
    O = Oracle()
    threads = os.cpu_count() or 1
    secs = []
    for s in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        r = O.process(p, ref_np, cor_np, W.points, order=order, neigh=neigh, n_process=n_sample,
                      seed_mode=0, n_threads=threads)
        if s >= args.warmup:
            secs.append(time.perf_counter() - t0)
    step_s = float(np.mean(secs))
    v = n_sample / step_s
    done = order[:n_sample]
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "points/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_s * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (the GPU arm's volumes: same generator and seeds)",
        "config": bench_config(W, world),
        "cpu_baseline": {"value": round(v, 4), "unit": "points/s", "cores": threads, "kind": "port",
                         "sample": f"the first {n_sample} points of the processing order per step, "
                                   "the reference's neighbour seeding, full search (grid + Gauss-Newton)"},
        "results": {"good": int((r["status"][done] == 0).sum()), "range_fail": int((r["status"][done] == -1).sum())},
        "e2e": {"value": round(v, 4), "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }))


if __name__ == "__main__":
    main()
