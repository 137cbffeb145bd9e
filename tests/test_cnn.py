"""The learned initial-guess network (dvc_cnn_*) and the learned search.

The network has no counterpart in the reference. Its FP64 oracle
(oracle/cnn_oracle.py) is pinned by a finite-difference check of its own
gradients (CPU); the GPU's patches, outputs and every weight gradient are
checked against the oracle (GPU); training must reduce the loss; and the
learned search (network start + Gauss-Newton + plain-search fallback) must
agree with the plain search.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import cnn_oracle as O


def test_oracle_gradients_by_finite_differences():
    rng = np.random.default_rng(0)
    lay, total = O.layout()
    p = np.zeros(total)
    for shape, w, b in lay:
        fan_in = int(np.prod(shape[1:]))
        p[w:w + int(np.prod(shape))] = rng.normal(0, np.sqrt(2.0 / fan_in), int(np.prod(shape)))
        p[b:b + shape[0]] = rng.normal(0, 0.05, shape[0])
    x = rng.normal(0, 1, (2, 2, 32, 32, 32))
    t = rng.normal(0, 1, (2, 12)) * O.SCALE
    loss, g = O.loss_and_grad(p, x, t)
    h = 1e-6
    checked = 0
    for shape, w, b in lay:  # a few weights and a bias of every layer
        for i in list(rng.choice(int(np.prod(shape)), 3, replace=False) + w) + [b]:
            pp, pm = p.copy(), p.copy()
            pp[i] += h
            pm[i] -= h
            fd = (O.loss_and_grad(pp, x, t)[0] - O.loss_and_grad(pm, x, t)[0]) / (2 * h)
            assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])
            checked += 1
    assert checked == 24


def _volumes(shape=(64, 64, 64), bpv=1):
    from digitalvolumecorrelation_gb300 import synth
    amp = (40.0, 200.0) if bpv == 1 else (2000.0, 60000.0)
    b = synth.blobs(shape, 260, amp=amp, seed=41)
    aff = synth.Affine(t=(1.2, -0.7, 0.5), E=((0.004, 0, 0), (0, -0.003, 0), (0, 0, 0.002)),
                       c=tuple(s / 2 for s in shape))
    dt = np.uint8 if bpv == 1 else np.uint16
    ns = 2.0 if bpv == 1 else 150.0
    ref = synth.render(shape, b, noise_sigma=ns, noise_seed=42, dtype=dt)
    cor = synth.render(shape, b, deform=aff, noise_sigma=ns, noise_seed=43, dtype=dt)
    return ref, cor, aff


def _he_weights(seed):
    rng = np.random.default_rng(seed)
    lay, total = O.layout()
    p = np.zeros(total, np.float32)
    for shape, w, b in lay:
        fan_in = int(np.prod(shape[1:]))
        p[w:w + int(np.prod(shape))] = rng.normal(0, np.sqrt(2.0 / fan_in), int(np.prod(shape)))
        p[b:b + shape[0]] = rng.normal(0, 0.05, shape[0])
    return p


@pytest.mark.gpu
@pytest.mark.parametrize("bpv", [1, 2])
def test_patches_vs_oracle(bpv):
    import torch
    from digitalvolumecorrelation_gb300 import engine
    from digitalvolumecorrelation_gb300.abi import make_params
    ref, cor, _ = _volumes(bpv=bpv)
    E = engine.Engine(make_params((64, 64, 64), bytes_per_voxel=bpv, subvol_size=11, subvol_npts=200,
                                  disp_max=3), ref, cor)
    pts = np.array([[32.0, 32.0, 32.0], [10.4, 50.6, 31.5], [3.0, 61.0, 60.2], [40.2, 20.7, 8.9]])
    pd = torch.from_numpy(pts).cuda()
    out = torch.zeros((len(pts), 2, 32, 32, 32), dtype=torch.float32, device="cuda")
    engine.Cnn.patches(E, len(pts), pd, out)
    got = out.cpu().numpy()
    for i, p in enumerate(pts):
        np.testing.assert_allclose(got[i, 0], O.patch(ref, p), atol=2e-4)
        np.testing.assert_allclose(got[i, 1], O.patch(cor, p), atol=2e-4)
    E.close()


def _grad_case():
    rng = np.random.default_rng(3)
    ref, cor, aff = _volumes()
    x = np.stack([np.stack([O.patch(ref, p), O.patch(cor, p)])
                  for p in rng.uniform(16, 48, (3, 3))]).astype(np.float32)
    t = (rng.normal(0, 1, (3, 12)) * O.SCALE).astype(np.float32)
    return x, t, _he_weights(5)


@pytest.mark.gpu
def test_fp32_kernels_forward_and_gradients_vs_oracle(monkeypatch):
    """The FP32 CUDA-core convolutions (DVC_CNN_FP32) and every backward
    kernel against the FP64 oracle: outputs within 1e-4, each layer's weight
    and bias gradients within 1e-3 of their scale."""
    import torch
    from digitalvolumecorrelation_gb300 import engine
    monkeypatch.setenv("DVC_CNN_FP32", "1")
    x, t, p = _grad_case()
    net = engine.Cnn(seed=1)
    net.set_weights(p)
    xd = torch.from_numpy(x).cuda()
    td = torch.from_numpy(t).cuda()
    y = torch.zeros((3, 12), dtype=torch.float32, device="cuda")
    net.forward(3, xd, y)
    y_ref, _, _, _ = O.forward(p.astype(np.float64), x)
    np.testing.assert_allclose(y.cpu().numpy(), y_ref, rtol=1e-4, atol=1e-4 * np.abs(y_ref).max())
    g, loss = net.gradients(3, xd, td)
    loss_ref, g_ref = O.loss_and_grad(p.astype(np.float64), x, t)
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref
    lay, _ = O.layout()
    for shape, w, b in lay:  # every layer's weights and biases
        for lo, n in ((w, int(np.prod(shape))), (b, shape[0])):
            a, r = g[lo:lo + n], g_ref[lo:lo + n]
            scale = np.abs(r).max()
            assert np.abs(a - r).max() <= 1e-3 * scale + 1e-9, (shape, np.abs(a - r).max(), scale)
    net.close()


@pytest.mark.gpu
def test_tensor_core_forward_and_gradients_vs_oracle():
    """The production path: convolutions on the tensor cores with BF16
    operands and FP32 sums. Against the oracle with the same operands rounded
    to BF16 the outputs agree to FP32 summation (rtol 1e-3); against the FP64
    network itself to the operands' BF16 rounding (3e-2). Gradients (FP32
    backward kernels over the BF16 forward's activations) against the oracle's
    of the same BF16 forward: rounding a forward activation to BF16 is
    discontinuous and near zero its ReLU mask can go either way, which moves
    single terms of a gradient (rounding alone moves these gradients by 6-18%
    of their scale against the FP64 network's), so the check is the
    direction of every layer's gradient (cosine >= 0.995) and 99% of its
    entries within 5% of its scale (the first layer's entries collect every
    downstream mask decision and move by 1-3%; the FP32 test above pins the
    backward kernels themselves to 1e-3)."""
    import torch
    from digitalvolumecorrelation_gb300 import engine
    x, t, p = _grad_case()
    net = engine.Cnn(seed=1)
    net.set_weights(p)
    xd = torch.from_numpy(x).cuda()
    td = torch.from_numpy(t).cuda()
    y = torch.zeros((3, 12), dtype=torch.float32, device="cuda")
    net.forward(3, xd, y)
    y_bf, _, _, _ = O.forward(p.astype(np.float64), x, bf16_convs=True)
    y_ref, _, _, _ = O.forward(p.astype(np.float64), x)
    yg = y.cpu().numpy()
    np.testing.assert_allclose(yg, y_bf, rtol=1e-3, atol=1e-3 * np.abs(y_bf).max())
    np.testing.assert_allclose(yg, y_ref, rtol=3e-2, atol=3e-2 * np.abs(y_ref).max())
    g, loss = net.gradients(3, xd, td)
    loss_ref, g_ref = O.loss_and_grad(p.astype(np.float64), x, t, bf16_convs=True)
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref
    lay, _ = O.layout()
    for shape, w, b in lay:
        n = int(np.prod(shape))
        a, r = g[w:w + n].astype(np.float64), g_ref[w:w + n]
        cos = a @ r / (np.linalg.norm(a) * np.linalg.norm(r))
        assert cos >= 0.995, (shape, cos)
        q99 = np.quantile(np.abs(a - r), 0.99)
        assert q99 <= 5e-2 * np.abs(r).max(), (shape, q99, np.abs(r).max())
    net.close()


@pytest.mark.gpu
def test_tensor_core_forward_many_tiles():
    """A batch of 40 patches: the first convolution has 1280 tiles of 128
    output voxels (several per CTA), the last ends in a partial tile; every
    output against the oracle with the convolutions' operands in BF16."""
    import torch
    from digitalvolumecorrelation_gb300 import engine
    rng = np.random.default_rng(11)
    x = rng.normal(0, 1, (40, 2, 32, 32, 32)).astype(np.float32)
    p = _he_weights(9)
    net = engine.Cnn(seed=1)
    net.set_weights(p)
    y = torch.zeros((40, 12), dtype=torch.float32, device="cuda")
    net.forward(40, torch.from_numpy(x).cuda(), y)
    y_bf, _, _, _ = O.forward(p.astype(np.float64), x, bf16_convs=True)
    np.testing.assert_allclose(y.cpu().numpy(), y_bf, rtol=1e-3, atol=1e-3 * np.abs(y_bf).max())
    net.close()


@pytest.mark.gpu
def test_training_reduces_loss():
    """Adam on patches of an affine pair with their true (u, v, w) as targets."""
    import torch
    from digitalvolumecorrelation_gb300 import engine
    from digitalvolumecorrelation_gb300.abi import make_params
    ref, cor, aff = _volumes()
    E = engine.Engine(make_params((64, 64, 64), subvol_size=11, subvol_npts=200, disp_max=3), ref, cor)
    rng = np.random.default_rng(8)
    pts = rng.uniform(14, 50, (64, 3))
    tgt = np.zeros((64, 12), np.float32)
    tgt[:, :3] = aff.u(pts)
    pd = torch.from_numpy(pts).cuda()
    x = torch.zeros((64, 2, 32, 32, 32), dtype=torch.float32, device="cuda")
    engine.Cnn.patches(E, 64, pd, x)
    td = torch.from_numpy(tgt).cuda()
    net = engine.Cnn(seed=2)
    first = net.train_step(64, x, td, 1e-3)
    for _ in range(150):
        last = net.train_step(64, x, td, 1e-3)
    assert last < 0.2 * first, (first, last)
    net.close()
    E.close()


@pytest.mark.gpu
def test_learned_search_and_fallback():
    """A network with zero weights proposes zero start parameters. Every point
    falling back (threshold -1) must give exactly the plain search seeded at
    zero (the rigid seed); with a real threshold the converged points agree
    with it within 0.01 voxel."""
    import torch
    from digitalvolumecorrelation_gb300 import engine
    from digitalvolumecorrelation_gb300.abi import make_params
    from digitalvolumecorrelation_gb300 import synth
    ref, cor, aff = _volumes()
    p = make_params((64, 64, 64), subvol_geom="cube", subvol_size=13, subvol_npts=400, num_srch_dof=6,
                    disp_max=3, basin_radius=1.5)
    E = engine.Engine(p, ref, cor)
    pts = synth.grid_points((3, 3, 3), 7.0, (32.0, 32.0, 32.0))
    n = len(pts)
    plain = E.process(pts, seed_mode=engine.SEED_RIGID)
    net = engine.Cnn(seed=3)
    net.set_weights(np.zeros(net.n_params, np.float32))
    dev = "cuda"
    pd = torch.from_numpy(pts).to(dev)
    od = torch.arange(n, dtype=torch.int32, device=dev)
    for thr, exact in ((-1.0, True), (0.1, False)):
        st = torch.empty(n, dtype=torch.int32, device=dev)
        ob = torch.empty(n, dtype=torch.float64, device=dev)
        pa = torch.empty((n, 12), dtype=torch.float64, device=dev)
        nfb = E.process_learned(net, n, pd, od, n, thr, st, ob, pa)
        s, o, q = st.cpu().numpy(), ob.cpu().numpy(), pa.cpu().numpy()
        good = (s == 0) & (plain["status"] == 0)
        if exact:
            assert nfb == n
            np.testing.assert_array_equal(s, plain["status"])
            np.testing.assert_array_equal(q, plain["params"])
            np.testing.assert_array_equal(o, plain["objmin"])
        else:
            assert good.sum() >= n - 2
            assert np.abs(q[good, :3] - plain["params"][good, :3]).max() <= 0.01
    net.close()
    E.close()


@pytest.mark.gpu
def test_learned_search_does_not_depend_on_point_order():
    """The learned search takes its points in locality order (a counting sort
    by the Morton code of each point's cell): every point's patch, network
    proposal and search are its own, so the same points given in any order
    (and a subset) give the same bits."""
    import torch
    from digitalvolumecorrelation_gb300 import engine, synth
    from digitalvolumecorrelation_gb300.abi import make_params
    ref, cor, aff = _volumes()
    p = make_params((64, 64, 64), subvol_geom="cube", subvol_size=13, subvol_npts=400, num_srch_dof=6,
                    disp_max=3, basin_radius=1.5)
    E = engine.Engine(p, ref, cor)
    rng = np.random.default_rng(7)
    pts = synth.grid_points((4, 4, 4), 5.0, (32.0, 32.0, 32.0)) + rng.normal(0.0, 0.3, (64, 3))
    n = len(pts)
    net = engine.Cnn(seed=5)
    # distinct proposals per point, near zero (within Gauss-Newton's reach)
    net.set_weights(net.get_weights() * np.float32(0.05))
    dev = "cuda"
    pd = torch.from_numpy(pts).to(dev)
    runs = []
    perm = rng.permutation(n).astype(np.int32)
    for order in (np.arange(n, dtype=np.int32), perm, perm[: n // 2].copy()):
        st = torch.empty(n, dtype=torch.int32, device=dev)
        ob = torch.empty(n, dtype=torch.float64, device=dev)
        pa = torch.empty((n, 12), dtype=torch.float64, device=dev)
        od = torch.from_numpy(order).to(dev)
        E.process_learned(net, n, pd, od, len(order), 10.0, st, ob, pa)
        runs.append((order, st.cpu().numpy(), ob.cpu().numpy(), pa.cpu().numpy()))
    (_, s0, o0, q0), (_, s1, o1, q1), (sub, s2, o2, q2) = runs
    assert (s0 == 0).sum() >= n // 2
    np.testing.assert_array_equal(s1, s0)
    np.testing.assert_array_equal(o1, o0)
    np.testing.assert_array_equal(q1, q0)
    np.testing.assert_array_equal(s2[sub], s0[sub])
    np.testing.assert_array_equal(q2[sub], q0[sub])
    rest = np.setdiff1d(np.arange(n), sub)
    assert np.all(s2[rest] == -3)  # not in the order: not searched
    net.close()
    E.close()


def _bump_pair(seed, shape=(96, 96, 96)):
    from digitalvolumecorrelation_gb300 import synth
    rng = np.random.default_rng(seed)
    field = synth.random_bumps(shape, rng, max_disp=4.0, max_strain=0.02, n_bumps=4)
    b = synth.blobs(shape, int(np.prod(shape)) // 300, seed=seed + 1)
    ref = synth.render(shape, b, noise_sigma=2.0, noise_seed=seed + 2)
    cor = synth.render(shape, b, deform=field, noise_sigma=2.0, noise_seed=seed + 3)
    return ref, cor, field


@pytest.mark.gpu
def test_trained_network_gains_over_the_plain_search(oracle):
    """What training buys. A network trained briefly on one pair (labels: the
    plain search's converged 12 parameters from the true translation)
    proposes each point's start on a held-out pair. The learned search
    (network start, Gauss-Newton, the plain search again where ZNSSD exceeds
    0.05) must need at most 40% of the plain search's objective evaluations
    (the plain search evaluates a 125-translation grid per point) and reach
    the FP64 oracle's optimum (within 0.01 voxel) as often as the plain
    search does; the same network untrained must gain nothing of that."""
    import torch
    from digitalvolumecorrelation_gb300 import engine, synth
    from digitalvolumecorrelation_gb300.abi import make_params
    shape = (96, 96, 96)
    kw = dict(subvol_geom="cube", subvol_size=17, subvol_npts=1000, obj_function="znssd",
              interp_type="tricubic", num_srch_dof=12, disp_max=6, basin_radius=3.0)
    p = make_params(shape, **kw)
    p0 = make_params(shape, **dict(kw, basin_radius=0.0))
    # training pair: labels from the true translation, Gauss-Newton only
    ref, cor, field = _bump_pair(61)
    tp = synth.grid_points((13, 13, 13), 4.0, (48.0, 48.0, 48.0))
    E0 = engine.Engine(p0, ref, cor)
    lab = E0.process(tp, seed_mode=engine.SEED_GIVEN, seeds=field.u(tp))
    keep = np.nonzero((lab["status"] == 0) & (lab["objmin"] < 0.05))[0].astype(np.int32)
    assert len(keep) > 1500
    net = engine.Cnn(seed=7)
    untrained = engine.Cnn(seed=7)
    dev = "cuda"
    tpd = torch.from_numpy(tp).to(dev)
    par = torch.from_numpy(lab["params"].astype(np.float32)).to(dev)
    x = torch.empty((64, 2, 32, 32, 32), dtype=torch.float32, device=dev)
    rng = np.random.default_rng(3)
    steps = 600
    for s in range(steps):
        pick = torch.from_numpy(rng.choice(keep, 64, replace=False)).to(dev)
        engine.Cnn.patches(E0, 64, tpd, x, idx_dev=pick)
        net.train_step(64, x, par.index_select(0, pick.long()).contiguous(),
                       1e-3 * 0.5 * (1.0 + np.cos(np.pi * s / steps)))
    E0.close()
    # held-out pair
    ref, cor, field = _bump_pair(71)
    pts = synth.grid_points((7, 7, 7), 8.0, (48.0, 48.0, 48.0))
    n = len(pts)
    order, neigh = oracle.order_neighbours(pts)
    E = engine.Engine(p, ref, cor)
    plain = E.process(pts, order=order, neigh=neigh)
    evals_plain = E.last_counters()[0]
    pd = torch.from_numpy(pts).to(dev)
    od = torch.from_numpy(order).to(dev)
    out = {}
    for name, nw in (("learned", net), ("untrained", untrained)):
        st = torch.empty(n, dtype=torch.int32, device=dev)
        ob = torch.empty(n, dtype=torch.float64, device=dev)
        pa = torch.empty((n, 12), dtype=torch.float64, device=dev)
        nfb = E.process_learned(nw, n, pd, od, n, 0.05, st, ob, pa)
        out[name] = dict(status=st.cpu().numpy(), params=pa.cpu().numpy(), fallback=nfb,
                         evals=E.last_counters()[0])
    E.close()
    # the FP64 oracle's optimum: Gauss-Newton from the true translation
    sample = np.arange(0, n, 7)
    o = oracle.process(p0, ref, cor, pts[sample], seed_mode=1, seeds=field.u(pts[sample]))
    ok = o["status"] == 0

    def within(st, pa):
        good = ok & (st[sample] == 0)
        err = np.abs(pa[sample][good, :3] - o["params"][good, :3]).max(axis=1)
        return int((err <= 0.01).sum())

    w_plain = within(plain["status"], plain["params"])
    w_learned = within(out["learned"]["status"], out["learned"]["params"])
    msg = (evals_plain, out["learned"]["evals"], out["untrained"]["evals"], out["learned"]["fallback"],
           out["untrained"]["fallback"], w_plain, w_learned, int(ok.sum()))
    assert out["learned"]["evals"] <= 0.4 * evals_plain, msg
    assert w_learned >= w_plain - 1, msg
    assert out["untrained"]["fallback"] >= 4 * max(1, out["learned"]["fallback"]), msg
    assert out["untrained"]["evals"] >= 2 * out["learned"]["evals"], msg
    net.close()
    untrained.close()
