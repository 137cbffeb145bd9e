"""FP64 restatement of the learned proposer network of libdvcgpu.so
(dvc_cnn.cu): forward pass, mean-squared-error loss and every weight gradient.

TEST INFRASTRUCTURE ONLY: the GPU network's outputs and gradients are checked
against this; nothing in the product imports it. The network has no
counterpart in the reference, so this oracle is pinned by its own
finite-difference gradient check (tests/test_cnn.py), not by reference data.

Layout (the library's): conv l has weights [Cout][Cin][3][3][3] (kz, ky, kx)
and Cout biases, then the dense layers [Nout][Nin] and Nout biases, all in one
flat vector; activations [B][C][z][y][x]; convolutions 3^3, stride 2, padding
1, ReLU; dense 768 -> 128 (ReLU) -> 12; outputs are the parameters divided by
SCALE.
"""
from __future__ import annotations

import numpy as np

CIN = [2, 16, 32, 64]
COUT = [16, 32, 64, 96]
DIN = [32, 16, 8, 4]
F0, F1, F2 = 768, 128, 12
SCALE = np.array([10.0, 10.0, 10.0, 0.05, 0.05, 0.05, 0.02, 0.02, 0.02, 0.02, 0.02, 0.02])


def layout():
    """[(weight shape, weight offset, bias offset)] of the flat parameter vector."""
    out, o = [], 0
    for ci, co in zip(CIN, COUT):
        out.append(((co, ci, 3, 3, 3), o, o + co * ci * 27))
        o += co * ci * 27 + co
    for nin, nout in ((F0, F1), (F1, F2)):
        out.append(((nout, nin), o, o + nout * nin))
        o += nout * nin + nout
    return out, o


def unpack(p):
    lay, total = layout()
    assert len(p) == total
    return [(p[w:w + int(np.prod(shape))].reshape(shape).astype(np.float64),
             p[b:b + shape[0]].astype(np.float64)) for shape, w, b in lay]


def _taps(Do):
    for kz in range(3):
        for ky in range(3):
            for kx in range(3):
                yield kz, ky, kx, (slice(kz, kz + 2 * Do, 2), slice(ky, ky + 2 * Do, 2), slice(kx, kx + 2 * Do, 2))


def conv_fwd(x, W, b):
    B, _, D = x.shape[:3]
    Do = D // 2
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1), (1, 1)))
    z = np.zeros((B, W.shape[0], Do, Do, Do)) + b[None, :, None, None, None]
    for kz, ky, kx, (sz, sy, sx) in _taps(Do):
        z += np.einsum("bcijk,oc->boijk", xp[:, :, sz, sy, sx], W[:, :, kz, ky, kx])
    return z


def conv_bwd(x, W, dz):
    """Gradients of z = conv(x) w.r.t. W, b and x, given dL/dz."""
    Do = dz.shape[2]
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1), (1, 1)))
    dW = np.zeros_like(W)
    dxp = np.zeros_like(xp)
    for kz, ky, kx, (sz, sy, sx) in _taps(Do):
        dW[:, :, kz, ky, kx] = np.einsum("boijk,bcijk->oc", dz, xp[:, :, sz, sy, sx])
        dxp[:, :, sz, sy, sx] += np.einsum("boijk,oc->bcijk", dz, W[:, :, kz, ky, kx])
    return dW, dz.sum(axis=(0, 2, 3, 4)), dxp[:, :, 1:-1, 1:-1, 1:-1]


def bf16(a):
    """Values rounded to bfloat16 (round to nearest, ties to even, through
    float32), returned as float64."""
    f = np.ascontiguousarray(np.asarray(a, np.float64).astype(np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(p, x, bf16_convs=False):
    """Outputs [B][12] and the activations (x: [B][2][32][32][32]).
    bf16_convs: every convolution's input and weights rounded to bfloat16
    first (the GPU's tensor-core convolutions; sums and biases exact here)."""
    layers = unpack(p)
    acts = [np.asarray(x, np.float64)]
    for W, b in layers[:4]:
        if bf16_convs:
            acts.append(np.maximum(conv_fwd(bf16(acts[-1]), bf16(W), b), 0.0))
        else:
            acts.append(np.maximum(conv_fwd(acts[-1], W, b), 0.0))
    h0 = acts[-1].reshape(len(x), -1)
    (W1, b1), (W2, b2) = layers[4], layers[5]
    h1 = np.maximum(h0 @ W1.T + b1, 0.0)
    y = h1 @ W2.T + b2
    return y, acts, h0, h1


def loss_and_grad(p, x, targets, bf16_convs=False):
    """Mean squared error of the scaled outputs against targets / SCALE, and
    the gradient w.r.t. the flat parameter vector. bf16_convs: the forward
    pass with bfloat16 convolutions (as `forward`), the backward pass exact
    with the unrounded weights and the activations that forward produced
    (the GPU's training step)."""
    y, acts, h0, h1 = forward(p, x, bf16_convs)
    B = len(x)
    e = y - np.asarray(targets, np.float64) / SCALE
    loss = np.mean(e * e)
    dy = 2.0 * e / (B * F2)
    layers = unpack(p)
    grads = [None] * 6
    (W1, _), (W2, _) = layers[4], layers[5]
    grads[5] = (dy.T @ h1, dy.sum(0))
    dh1 = (dy @ W2) * (h1 > 0)
    grads[4] = (dh1.T @ h0, dh1.sum(0))
    dz = ((dh1 @ W1) * (h0 > 0)).reshape(acts[4].shape)
    for l in range(3, -1, -1):
        dW, db, dx = conv_bwd(acts[l], layers[l][0], dz)
        grads[l] = (dW, db)
        if l > 0:
            dz = dx * (acts[l] > 0)
    lay, total = layout()
    g = np.zeros(total)
    for (shape, w, b), (dW, db) in zip(lay, grads):
        g[w:w + dW.size] = dW.ravel()
        g[b:b + db.size] = db
    return loss, g


def patch(vol_zyx, point):
    """32^3 patch of a volume [z][y][x] around round(point) (0 outside),
    normalised to zero mean and unit variance."""
    o = np.floor(np.asarray(point, np.float64) + 0.5).astype(int) - 16
    out = np.zeros((32, 32, 32))
    nz, ny, nx = vol_zyx.shape
    zs, ys, xs = [np.arange(o[d], o[d] + 32) for d in (2, 1, 0)]
    vz, vy, vx = (zs >= 0) & (zs < nz), (ys >= 0) & (ys < ny), (xs >= 0) & (xs < nx)
    out[np.ix_(vz, vy, vx)] = vol_zyx[np.ix_(zs[vz], ys[vy], xs[vx])]
    m = out.mean()
    return (out - m) / np.sqrt(((out - m) ** 2).mean() + 1e-6)
