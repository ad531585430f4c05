"""CPU restatement (numpy float32) of the patch-registration network's loss
and gradient -- test infrastructure only, the checker of the GPU kernels in
patchvvc-plus_gb300/csrc/regnet.cu and gemm_tcgen05.cu.

The network has no counterpart in the reference (which registers every patch
with PCL ICP from the identity, src/registration/icp.cc:21-102), so this is
not a restatement of reference code: it restates the model the GPU trains,
and rounds to bf16 (round to nearest even) exactly where the GPU stores bf16:
the activations X1, X2, Y3, H1, H2, the weight copies of W2..W5, and the
backward's dH2, dH1, dY2, dY1.  Sums are fp32 in numpy's order, so results
agree with the GPU up to fp32 reassociation (and the rare bf16 rounding flip
that reassociation causes).

Model (P = 256 points per cloud, rows of cloud c = 2*pair + side):
  X1 = relu(W1 x0 + b1)  (3->64, ((w0 x + w1 y) + w2 z) + b1 in fp32)
  X2 = relu(X1 W2^T + b2)  (64->128)      Y3 = relu(X2 W3^T + b3)  (128->256)
  H0 = [max_rows Y3(src) | max_rows Y3(tgt)]  (first maximum)
  H1 = relu(H0 W4^T + b4)  (512->256)     H2 = relu(H1 W5^T + b5)  (256->128)
  out = H2 W6^T + b6  (128->6)
  loss = sum_b sum_j w_j (out_bj - y_bj)^2 / B,  w = lambda_w for j < 3 else 1
"""
from __future__ import annotations

import numpy as np

P = 256
DIMS = dict(w1=(64, 3), b1=(64,), w2=(128, 64), b2=(128,), w3=(256, 128), b3=(256,), w4=(256, 512), b4=(256,),
            w5=(128, 256), b5=(128,), w6=(6, 128), b6=(6,))


def bf16(x: np.ndarray) -> np.ndarray:
    """float32 -> nearest bf16 (ties to even), returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    r = ((b >> 16) & 1) + 0x7FFF
    return ((b + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def unflatten(flat: np.ndarray) -> dict:
    out, o = {}, 0
    for k, shp in DIMS.items():
        n = int(np.prod(shp))
        out[k] = np.asarray(flat[o:o + n], np.float32).reshape(shp)
        o += n
    assert o == flat.size
    return out


def flatten(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[k], np.float32).reshape(-1) for k in DIMS])


def loss_and_grad(flat: np.ndarray, x0: np.ndarray, y: np.ndarray, lambda_w: float):
    """x0 [B,2,P,3] fp32 (pair b's source rows then target rows), y [B,6].
    Returns (loss, flat gradient, out [B,6])."""
    f32 = np.float32
    p = unflatten(np.asarray(flat, np.float32))
    B = y.shape[0]
    x0 = np.asarray(x0, f32).reshape(-1, 3)
    R = x0.shape[0]
    assert R == 2 * B * P
    W1, b1 = p["w1"], p["b1"]
    pre1 = ((x0[:, 0:1] * W1[:, 0] + x0[:, 1:2] * W1[:, 1]) + x0[:, 2:3] * W1[:, 2]) + b1
    X1 = bf16(np.maximum(pre1, f32(0)))
    W2b, W3b, W4b, W5b = bf16(p["w2"]), bf16(p["w3"]), bf16(p["w4"]), bf16(p["w5"])
    X2 = bf16(np.maximum(X1 @ W2b.T + p["b2"], f32(0)))
    Y3 = bf16(np.maximum(X2 @ W3b.T + p["b3"], f32(0)))
    Yc = Y3.reshape(2 * B, P, 256)
    amax = Yc.argmax(axis=1)                              # first maximum per (cloud, channel)
    G = np.take_along_axis(Yc, amax[:, None, :], axis=1)[:, 0, :]
    H0 = G.reshape(B, 512)
    H1 = bf16(np.maximum(H0 @ W4b.T + p["b4"], f32(0)))
    H2 = bf16(np.maximum(H1 @ W5b.T + p["b5"], f32(0)))
    out = H2 @ p["w6"].T + p["b6"]
    w = np.array([lambda_w] * 3 + [1.0] * 3, f32)
    e = out - y.astype(f32)
    loss = float((w * e * e).sum() / B)
    dout = (f32(2) * w * e / f32(B)).astype(f32)
    g = {k: np.zeros(s, f32) for k, s in DIMS.items()}
    g["w6"] = dout.T @ H2
    g["b6"] = dout.sum(0)
    dH2 = bf16((dout @ p["w6"]) * (H2 > 0))
    g["w5"] = dH2.T @ H1
    g["b5"] = dH2.sum(0)
    dH1 = bf16((dH2 @ W5b) * (H1 > 0))
    g["w4"] = dH1.T @ H0
    g["b4"] = dH1.sum(0)
    dH0 = (dH1 @ W4b).astype(f32)
    gp = np.where(H0 > 0, dH0, f32(0)).reshape(2 * B, 256)   # gradient reaching each pooled channel
    rows = (np.arange(2 * B)[:, None] * P + amax).reshape(-1)  # argmax row of every (cloud, channel)
    gflat = gp.reshape(-1)
    ch = np.tile(np.arange(256), 2 * B)
    g["w3"] = np.zeros((256, 128), f32)
    np.add.at(g["w3"], ch, gflat[:, None] * X2[rows])
    g["b3"] = gp.sum(0)
    dX2 = np.zeros((R, 128), f32)
    np.add.at(dX2, rows, gflat[:, None] * W3b[ch])
    dY2 = bf16(dX2 * (X2 > 0))
    g["w2"] = dY2.T @ X1
    g["b2"] = dY2.sum(0)
    dY1 = bf16((dY2 @ W2b) * (X1 > 0))
    g["w1"] = dY1.T @ x0
    g["b1"] = dY1.sum(0)
    return loss, flatten(g), out
