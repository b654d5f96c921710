"""FP64 numpy restatement of the surrogate network's forward and backward pass.

TEST INFRASTRUCTURE ONLY. This module is an oracle: the tests use it to
check the gradients that the GPU kernels (BF16 tensor-core GEMMs with FP32
accumulation) compute. The product never imports it.

The network (no counterpart in the reference, which has no learned part):
  x [B, H, W, Cin] (NHWC), slot [B] (each shot's source receiver slot)
  5 x { 3x3 stride-2 pad-1 conv + bias + ReLU }       channels `chans`
  flatten -> dense(latent) + ReLU                       -> h
  dense((2 nrec - 1) * modes)                           -> z (offset-trace coefficients)
  q[b, o, :] = z[b, o, :] @ basis [modes, nt]           (spectral synthesis)
  p[b, r, :] = q[b, r + nrec - 1 - slot[b], :]          (offset -> receiver)
  head: dense(1) on h, detached from the trunk          -> predicted log misfit
Loss = mean_b ||p_b - t_b||^2 / ||t_b||^2
     + head_weight * mean_b (head_b - log(loss_b))^2     (loss_b treated as data)

Weights follow the product's layout: conv W [Cout][9*Cin] with column
(ky*3 + kx)*Cin + c; dense W [out][in].
"""
from __future__ import annotations

import numpy as np


def im2col(x):
    """x [B, H, W, C] -> [B*Ho*Wo, 9*C]: 3x3 patches, stride 2, zero pad 1."""
    B, H, W, C = x.shape
    Ho, Wo = (H + 1) // 2, (W + 1) // 2
    xp = np.zeros((B, H + 2, W + 2, C), x.dtype)
    xp[:, 1:H + 1, 1:W + 1] = x
    cols = [xp[:, ky:ky + 2 * Ho:2, kx:kx + 2 * Wo:2, :] for ky in range(3) for kx in range(3)]
    return np.stack(cols, axis=3).reshape(B * Ho * Wo, 9 * C), (Ho, Wo)


def col2im(dcol, shape):
    """Adjoint of im2col: dcol [B*Ho*Wo, 9*C] -> dx [B, H, W, C]."""
    B, H, W, C = shape
    Ho, Wo = (H + 1) // 2, (W + 1) // 2
    d = dcol.reshape(B, Ho, Wo, 9, C)
    dxp = np.zeros((B, H + 2, W + 2, C), dcol.dtype)
    for ky in range(3):
        for kx in range(3):
            dxp[:, ky:ky + 2 * Ho:2, kx:kx + 2 * Wo:2, :] += d[:, :, :, ky * 3 + kx, :]
    return dxp[:, 1:H + 1, 1:W + 1]


def forward(params, x, slot, basis, nrec, modes):
    """params: dict of FP64 arrays conv{l}_w/b, fc1_w/b, fc2_w/b, head_w/b.
    Returns (p [B, nrec*nt], head [B], cache)."""
    cache = {"x": x}
    a = x
    nconv = sum(1 for k in params if k.startswith("conv") and k.endswith("_w"))
    for l in range(nconv):
        col, (Ho, Wo) = im2col(a)
        y = col @ params[f"conv{l}_w"].T + params[f"conv{l}_b"]
        cache[f"col{l}"], cache[f"shape{l}"] = col, a.shape
        cache[f"y{l}"] = y
        a = np.maximum(y, 0.0).reshape(a.shape[0], Ho, Wo, -1)
    B = x.shape[0]
    f = a.reshape(B, -1)
    cache["f"] = f
    y1 = f @ params["fc1_w"].T + params["fc1_b"]
    h = np.maximum(y1, 0.0)
    cache["fc1_y"], cache["h"] = y1, h
    z = h @ params["fc2_w"].T + params["fc2_b"]
    cache["z"] = z
    q = (z.reshape(-1, modes) @ basis).reshape(B, 2 * nrec - 1, -1)
    rows = np.arange(nrec)[None, :] + (nrec - 1 - np.asarray(slot))[:, None]
    p = np.take_along_axis(q, rows[:, :, None], axis=1).reshape(B, -1)
    cache["rows"] = rows
    head = (h @ params["head_w"].T + params["head_b"])[:, 0]
    return p, head, cache


def loss_and_grads(params, x, slot, target, basis, nrec, modes, head_weight):
    """Return (loss_b [B], head [B], grads dict) of the loss in the module docstring."""
    p, head, c = forward(params, x, slot, basis, nrec, modes)
    B = x.shape[0]
    t2 = np.sum(target * target, axis=1)
    r = p - target
    loss = np.sum(r * r, axis=1) / t2
    g = {}
    dp = 2.0 * r / t2[:, None] / B
    nt = basis.shape[1]
    dq = np.zeros((B, 2 * nrec - 1, nt))
    np.put_along_axis(dq, c["rows"][:, :, None], dp.reshape(B, nrec, nt), axis=1)
    dz = (dq.reshape(-1, nt) @ basis.T).reshape(B, -1)
    g["fc2_w"] = dz.T @ c["h"]
    g["fc2_b"] = dz.sum(0)
    dhead = 2.0 * head_weight * (head - np.log(np.maximum(loss, 1e-12))) / B
    g["head_w"] = dhead[None, :] @ c["h"]
    g["head_b"] = np.array([dhead.sum()])
    dh = dz @ params["fc2_w"]
    dy1 = dh * (c["fc1_y"] > 0)
    g["fc1_w"] = dy1.T @ c["f"]
    g["fc1_b"] = dy1.sum(0)
    df = dy1 @ params["fc1_w"]
    nconv = sum(1 for k in params if k.startswith("conv") and k.endswith("_w"))
    da = df
    for l in reversed(range(nconv)):
        y = c[f"y{l}"]
        dy = da.reshape(y.shape) * (y > 0)
        g[f"conv{l}_w"] = dy.T @ c[f"col{l}"]
        g[f"conv{l}_b"] = dy.sum(0)
        if l > 0:
            da = col2im(dy @ params[f"conv{l}_w"], c[f"shape{l}"])
    return loss, head, g


def total_loss(params, x, slot, target, basis, nrec, modes, head_weight):
    """Mean squared relative misfit (the trunk's objective), the head and the
    per-shot misfits."""
    p, head, _ = forward(params, x, slot, basis, nrec, modes)
    t2 = np.sum(target * target, axis=1)
    loss = np.sum((p - target) ** 2, axis=1) / t2
    return float(np.mean(loss)), head, loss
