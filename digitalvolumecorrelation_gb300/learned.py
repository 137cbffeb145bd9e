"""Configuration 4: the learned initial guess, trained and judged on the GPU.

Training pairs are 512^3 uint8 speckle volumes (one Gaussian blob per 1000
voxels, sigma 1.5-3 voxels, amplitude 40-200, noise sigma 2) whose correlate
volume is deformed by a random smooth field (translation, uniform strain of up
to 2%, Gaussian bumps; |u| < 10 voxels, `synth.random_bumps`). Training
points lie on a grid of spacing 12 voxels (five pairs, about 250,000 labelled
patch pairs for the configuration's 200,000), held-out points on one of
spacing 16. Labels are the 12 parameters the plain GPU
search converges to from the true translation (no coarse grid needed there);
points that do not converge well are left out. The network (dvc_cnn_*) is
trained by Adam on patches cut on the fly from the resident volumes.

`evaluate` then runs, on a held-out pair, the plain GPU method (reference
seeding, coarse grid over disp_max 10, Gauss-Newton) at two grid resolutions
(basin radius 2.5: 9^3 = 729 translations; basin radius 5: 5^3 = 125) and
the learned method (network start, Gauss-Newton, plain search for points whose
ZNSSD exceeds the threshold) and times each; bench.py checks them against the
FP64 oracle on a sample of points.

    python -m digitalvolumecorrelation_gb300.learned [--steps N]
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

from . import engine, synth, workloads
from .abi import make_params

SHAPE = (512, 512, 512)
SEARCH = dict(subvol_geom="cube", subvol_size=31, subvol_npts=2000, obj_function="znssd",
              interp_type="tricubic", num_srch_dof=12, disp_max=10, basin_radius=2.5)
SPACING = 16.0        # held-out points
TRAIN_SPACING = 12.0  # training points
TRAIN_PAIRS = 5
COARSE_BASIN = 5.0    # the second plain method: disp_max / 2, a 125-translation grid
MARGIN = 40.0
OBJ_THRESHOLD = 0.05


def grid(shape=SHAPE, spacing=SPACING, margin=MARGIN):
    n = [int((s - 2 * margin) // spacing) + 1 for s in shape]
    centre = [margin + (m - 1) * spacing / 2.0 for m in n]
    return synth.grid_points(tuple(n), spacing, tuple(centre))


class Pair:
    """One rendered pair resident on the GPU, its deformation and ROI points."""

    def __init__(self, seed, shape=SHAPE, spacing=SPACING):
        import torch
        rng = np.random.default_rng(seed)
        self.deform = synth.random_bumps(shape, rng)
        nvox = int(np.prod(shape))
        self.blobs = synth.blobs(shape, nvox // 1000, sigma=(1.5, 3.0), amp=(40.0, 200.0), seed=seed + 7)
        self.w = workloads.Workload(f"config4_pair{seed}", shape, 1, SEARCH, grid(shape, spacing), self.deform,
                                    self.blobs, 2.0, seed + 11, seed + 13)
        self.ref, self.cor = self.w.render_device()
        self.points = self.w.points
        self.truth = self.deform.u(self.points)
        self.pts_dev = torch.from_numpy(self.points).cuda()

    def engine(self, **over):
        kw = dict(SEARCH, **over)
        return engine.Engine(make_params(self.w.shape, **kw), ref_dev=self.ref, cor_dev=self.cor)


def labels(pair):
    """Plain-search converged parameters from the true translation; rows kept."""
    E = pair.engine(basin_radius=0.0)
    r = E.process(pair.points, seed_mode=engine.SEED_GIVEN, seeds=pair.truth)
    E.close()
    keep = (r["status"] == 0) & (r["objmin"] < OBJ_THRESHOLD)
    return r["params"].astype(np.float32), keep


def train(pairs, steps=2000, batch=256, lr=1e-3, seed=1, log=None):
    """Adam on random batches (one pair per batch); cosine learning rate."""
    import torch
    net = engine.Cnn(seed=seed)
    rng = np.random.default_rng(seed)
    data = []
    for p in pairs:
        par, keep = labels(p)
        idx = np.nonzero(keep)[0].astype(np.int32)
        data.append((p, p.engine(), torch.from_numpy(par).cuda(), idx))
    x = torch.empty((batch, 2, 32, 32, 32), dtype=torch.float32, device="cuda")
    losses = []
    t0 = time.perf_counter()
    for s in range(steps):
        p, E, par, idx = data[s % len(data)]
        pick = torch.from_numpy(rng.choice(idx, batch, replace=False)).cuda()
        engine.Cnn.patches(E, batch, p.pts_dev, x, idx_dev=pick)
        t = par.index_select(0, pick.long()).contiguous()
        lr_s = lr * 0.5 * (1.0 + np.cos(np.pi * s / steps))
        losses.append(net.train_step(batch, x, t, lr_s))
        if log and (s % 250 == 0 or s == steps - 1):
            log(f"step {s} loss {np.mean(losses[-50:]):.5f}")
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    for _, E, _, _ in data:
        E.close()
    n_train = int(sum(len(d[3]) for d in data))
    return net, dict(steps=steps, batch=batch, seconds=secs, samples=n_train,
                     loss_first=float(np.mean(losses[:20])), loss_last=float(np.mean(losses[-50:])))


def _time(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def proposal_error(net, pair, batch=1024):
    """RMS error of the network's proposals against the labels, per parameter
    (held-out pair, converged points)."""
    import torch
    par, keep = labels(pair)
    idx = np.nonzero(keep)[0].astype(np.int32)
    E = pair.engine()
    x = torch.empty((batch, 2, 32, 32, 32), dtype=torch.float32, device="cuda")
    y = torch.empty((batch, 12), dtype=torch.float32, device="cuda")
    pred = np.zeros((len(idx), 12))
    for r0 in range(0, len(idx), batch):
        nb = min(batch, len(idx) - r0)
        sel = torch.from_numpy(idx[r0:r0 + nb]).cuda()
        engine.Cnn.patches(E, nb, pair.pts_dev, x, idx_dev=sel)
        net.forward(nb, x, y)
        pred[r0:r0 + nb] = y[:nb].cpu().numpy() * SCALE
    E.close()
    return np.sqrt(np.mean((pred - par[idx]) ** 2, axis=0))


SCALE = np.array([10.0, 10.0, 10.0, 0.05, 0.05, 0.05, 0.02, 0.02, 0.02, 0.02, 0.02, 0.02])


def evaluate(net, pair):
    """Plain vs learned on a held-out pair: throughput, convergence, error
    against the true field. Returns the summary and, per method, the status and
    parameter arrays (for checks against the FP64 oracle, done by the caller)."""
    import torch
    n = len(pair.points)
    order, neigh = workloads.order_and_neighbours(pair.points)
    dev = "cuda"
    od = torch.from_numpy(order).to(dev)
    nd = torch.from_numpy(neigh).to(dev)
    out = {}
    E = pair.engine()
    E125 = pair.engine(basin_radius=COARSE_BASIN)
    res = {}
    for name in ("plain", "plain_125", "learned"):
        st = torch.empty(n, dtype=torch.int32, device=dev)
        ob = torch.empty(n, dtype=torch.float64, device=dev)
        pa = torch.empty((n, 12), dtype=torch.float64, device=dev)
        it = torch.empty(n, dtype=torch.int32, device=dev)
        if name == "plain":
            run = lambda: E.process_device(n, pair.pts_dev, od, n, nd, neigh.shape[1], engine.SEED_NEIGHBOURS,
                                           None, st, ob, pa, it)
        elif name == "plain_125":
            run = lambda: E125.process_device(n, pair.pts_dev, od, n, nd, neigh.shape[1], engine.SEED_NEIGHBOURS,
                                              None, st, ob, pa, it)
        else:
            run = lambda: E.process_learned(net, n, pair.pts_dev, od, n, OBJ_THRESHOLD, st, ob, pa, it)
        run()  # warm-up
        fb, secs = _time(run)
        evals = (E125 if name == "plain_125" else E).last_counters()[0]
        res[name] = (st.cpu().numpy(), pa.cpu().numpy())
        out[name] = dict(points_per_s=round(n / secs, 1), seconds=round(secs, 4),
                         good=int((res[name][0] == 0).sum()), evaluations=evals,
                         mean_gn_iterations=float(it.float().mean().item()))
        if name == "learned":
            out[name]["fallback_points"] = int(fb)
        else:
            k = int(SEARCH["disp_max"] / (COARSE_BASIN if name == "plain_125" else SEARCH["basin_radius"]))
            out[name]["grid_translations"] = (2 * k + 1) ** 3
    E.close()
    E125.close()
    for name in ("plain", "plain_125", "learned"):
        s, pa = res[name]
        out[name]["max_err_vs_truth_vox"] = float(np.abs(pa[s == 0, :3] - pair.truth[s == 0]).max())
    out["speedup_learned_over_plain"] = round(out["learned"]["points_per_s"] / out["plain"]["points_per_s"], 2)
    out["speedup_learned_over_plain_125"] = round(out["learned"]["points_per_s"] / out["plain_125"]["points_per_s"], 2)
    return out, res


def run(steps=3000, train_pairs=TRAIN_PAIRS, log=None, keep=False):
    """Train on `train_pairs` pairs, evaluate on a held-out one. With keep,
    also return the held-out pair, the per-method results and the trained
    weights."""
    pairs = [Pair(101 + 17 * k, spacing=TRAIN_SPACING) for k in range(train_pairs)]
    net, tinfo = train(pairs, steps=steps, log=log)
    for p in pairs:
        del p.ref, p.cor
    held = Pair(9001)
    rms = proposal_error(net, held)
    ev, res = evaluate(net, held)
    ev["proposal_rms"] = {"uvw_vox": [round(float(v), 4) for v in rms[:3]],
                          "rotation_rad": [round(float(v), 5) for v in rms[3:6]],
                          "strain": [round(float(v), 5) for v in rms[6:]]}
    weights = net.get_weights()
    net.close()
    summary = dict(config="config4_512cube_u8_bumps_cube31_dof12", search=SEARCH, spacing=SPACING,
                   points=len(held.points), obj_threshold=OBJ_THRESHOLD, training=tinfo, **ev)
    return (summary, held, res, weights) if keep else summary


if __name__ == "__main__":
    steps = int(sys.argv[sys.argv.index("--steps") + 1]) if "--steps" in sys.argv else 3000
    print(json.dumps(run(steps=steps, log=lambda m: print(m, file=sys.stderr))))
