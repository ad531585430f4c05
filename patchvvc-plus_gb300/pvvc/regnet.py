"""Learned ICP initialisation over the C ABI (pvvc_regnet_*, pvvc_propose).

A PointNet-style network maps a (source, target) patch pair to an initial
rigid transform for pvvc_icp_batch.  The reference has no counterpart: it
starts every registration from the identity (src/registration/icp.cc:21-102).
Training labels are the transforms plain ICP converges to.  A proposal only
seeds ICP: `register_learned` refines it with a few ICP iterations and hands
every pair whose refinement did not converge to plain ICP from the identity
(or, with judge="plain", keeps a refined result only where its MSE is no
worse than plain ICP's).  The registration is still an ICP result, so the
motion vectors and the bitstream the encoder writes are of the kind the
reference decoder reads.

Device buffers are torch tensors (plumbing only); the network's kernels
(sampling, tcgen05 GEMMs, pooling, backward, AdamW) run in libpvvc_gb300.so."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

P = 256  # points sampled per cloud
DIMS = dict(w1=(64, 3), b1=(64,), w2=(128, 64), b2=(128,), w3=(256, 128), b3=(256,), w4=(256, 512), b4=(256,),
            w5=(128, 256), b5=(128,), w6=(6, 128), b6=(6,))


class AdamW(C.Structure):
    _fields_ = [("lr", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
                ("weight_decay", C.c_float), ("lambda_w", C.c_float)]


def unflatten(flat: np.ndarray) -> dict:
    """The flat fp32 parameter vector as named arrays (layout of regnet.cu)."""
    out, o = {}, 0
    for k, shp in DIMS.items():
        n = int(np.prod(shp))
        out[k] = flat[o:o + n].reshape(shp)
        o += n
    assert o == flat.size
    return out


def axis_angle(R: np.ndarray) -> np.ndarray:
    """log map of rotation matrices [n,3,3] -> axis-angle [n,3] (float64)."""
    R = np.asarray(R, np.float64)
    c = np.clip((np.trace(R, axis1=1, axis2=2) - 1) / 2, -1, 1)
    th = np.arccos(c)
    w = np.stack([R[:, 2, 1] - R[:, 1, 2], R[:, 0, 2] - R[:, 2, 0], R[:, 1, 0] - R[:, 0, 1]], 1)
    s = np.sin(th)
    k = np.where(s[:, None] > 1e-9, w / (2 * np.where(s > 1e-9, s, 1))[:, None], 0.5 * w)
    return k * th[:, None]


class RegNet:
    """One network (fp32 master parameters, AdamW state, bf16 copies) on the
    current CUDA device."""

    def __init__(self, seed: int = 0):
        self.h = C.c_void_p()
        L.check(L.lib().pvvc_regnet_create(seed, C.byref(self.h)), "pvvc_regnet_create")
        self.nparam = int(L.lib().pvvc_regnet_param_count())

    def close(self):
        if self.h:
            L.lib().pvvc_regnet_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.nparam, np.float32)
        L.check(L.lib().pvvc_regnet_get_params(self.h, out.ctypes.data_as(L.f32p), self.nparam), "get_params")
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        L.check(L.lib().pvvc_regnet_set_params(self.h, p.ctypes.data_as(L.f32p), self.nparam), "set_params")

    def grad(self, x0, y, lambda_w: float, stream: int = 0):
        """Gradient and loss for normalised inputs x0 (device [B,2,P,3] fp32)
        and targets y (device [B,6]); no update.  Returns device tensors."""
        import torch
        B = int(y.shape[0])
        g = torch.empty(self.nparam, dtype=torch.float32, device=y.device)
        loss = torch.empty(1, dtype=torch.float32, device=y.device)
        L.check(L.lib().pvvc_regnet_grad(self.h, B, x0.data_ptr(), y.data_ptr(), lambda_w, g.data_ptr(), loss.data_ptr(),
                                         stream), "pvvc_regnet_grad")
        return g, loss

    def train_step(self, data: "PairData", ids, seed: int, opt: AdamW, loss_out=None, stream: int = 0) -> None:
        """One AdamW step on pairs `ids` (device int32) of a labelled dataset."""
        L.check(L.lib().pvvc_regnet_train_step(self.h, int(ids.numel()), ids.data_ptr(), data.src.data_ptr(),
                                               data.soff.data_ptr(), data.tgt.data_ptr(), data.toff.data_ptr(),
                                               data.T_label.data_ptr(), data.omega_label.data_ptr(), seed, C.byref(opt),
                                               None if loss_out is None else loss_out.data_ptr(), stream),
                "pvvc_regnet_train_step")

    def propose(self, data, seed: int = 0, T_out=None, stream: int = 0):
        """Proposed initial transforms (device [n,16] row-major) for every pair."""
        import torch
        if T_out is None:
            T_out = torch.empty((data.n, 16), dtype=torch.float32, device=data.src.device)
        L.check(L.lib().pvvc_propose(self.h, data.n, data.src.data_ptr(), data.soff.data_ptr(), data.tgt.data_ptr(),
                                     data.toff.data_ptr(), seed, T_out.data_ptr(), stream), "pvvc_propose")
        return T_out

    def outputs(self, n: int, stream: int = 0):
        import torch
        out = torch.empty((n, 6), dtype=torch.float32, device="cuda")
        L.check(L.lib().pvvc_regnet_outputs(self.h, n, out.data_ptr(), stream), "pvvc_regnet_outputs")
        return out


class PairData:
    """Device-resident pairs (the IcpBatch layout) with optional labels."""

    def __init__(self, icp_batch, T_label: np.ndarray | None = None):
        self._init(icp_batch.src, icp_batch.soff, icp_batch.tgt, icp_batch.toff, T_label)

    @classmethod
    def from_packed(cls, src, soff, tgt, toff, T_label: np.ndarray | None = None) -> "PairData":
        d = cls.__new__(cls)
        d._init(src, soff, tgt, toff, T_label)
        return d

    def _init(self, src, soff, tgt, toff, T_label):
        import torch
        self.n = int(soff.numel()) - 1
        self.src, self.soff, self.tgt, self.toff = src, soff, tgt, toff
        if T_label is not None:
            T = np.asarray(T_label, np.float32).reshape(-1, 4, 4)
            self.T_label = torch.from_numpy(T.reshape(-1, 16).copy()).to(self.src.device)
            self.omega_label = torch.from_numpy(axis_angle(T[:, :3, :3]).astype(np.float32)).to(self.src.device)


def subset_batch(b, idx):
    """An IcpBatch of the pairs `idx` (device int64) of batch b, gathered on
    the device."""
    import torch

    from .icp import IcpBatch
    so, to = b.soff.long(), b.toff.long()
    ns, nt = so[1:] - so[:-1], to[1:] - to[:-1]
    s_n, t_n = ns[idx], nt[idx]

    def gather(pts, off, n):
        o = torch.cat([torch.zeros(1, dtype=torch.int64, device=pts.device), torch.cumsum(n, 0)])
        own = torch.repeat_interleave(torch.arange(idx.numel(), device=pts.device), n)
        loc = torch.arange(int(o[-1]), device=pts.device) - o[:-1][own]
        return pts[off[idx][own] + loc], o.to(torch.int32)

    src, nso = gather(b.src, so, s_n)
    tgt, nto = gather(b.tgt, to, t_n)
    return IcpBatch(None, packed=(src, nso, tgt, nto))


def register_learned(net: RegNet, b, refine_iters: int = 10, accept_rel: float = 1e-3, judge: str = "converged",
                     seed: int = 0, plain=None):
    """Registration of every pair of IcpBatch b with a learned initial guess.

    The network proposes T0 (pvvc_propose); ICP refines it for at most
    `refine_iters` iterations and reports convergence when the relative
    change of the MSE falls below `accept_rel`.  judge="converged": a pair
    keeps its refined result if that ICP converged, otherwise plain ICP from
    the identity (50 iterations, the encoder's default) registers it.
    judge="plain": plain ICP is run for every pair as well (`plain` = its
    (T, mse) if already computed) and a pair keeps the refined result only if
    its MSE is no worse.  judge="tight": ICP refines the proposal to plain
    ICP's own stopping rule (at most 50 iterations, |dMSE| < 1e-6), with no
    fallback.  Returns device tensors (T [n,16], mse [n]) and
    {"fallback": pairs registered by plain ICP, "accepted": device bool [n]}."""
    import torch
    data = PairData(b)
    T0 = net.propose(data, seed=seed, stream=torch.cuda.current_stream().cuda_stream)
    if judge == "tight":
        # ICP from the proposal to plain ICP's own stopping rule (at most 50
        # iterations, |dMSE| < 1e-6): both runs end in a converged ICP minimum
        b.run(init=T0, max_iter=50, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)
        return b.T.clone(), b.mse.clone(), {"fallback": 0, "accepted": b.conv.clone().bool()}
    b.run(init=T0, max_iter=refine_iters, fitness_eps=accept_rel, transform_eps=0.0, mse_abs_eps=1e-6)
    T = b.T.clone()
    mse = b.mse.clone()
    conv = b.conv.clone().bool()
    if judge == "plain":
        if plain is None:
            b.run(max_iter=50, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)
            plain = (b.T.clone(), b.mse.clone())
        worse = mse > plain[1]
        T = torch.where(worse[:, None], plain[0], T)
        mse = torch.where(worse, plain[1], mse)
        return T, mse, {"fallback": int(worse.sum()), "accepted": ~worse}
    rej = torch.nonzero(~conv).squeeze(1)
    nrej = int(rej.numel())
    if nrej:
        sb = subset_batch(b, rej)
        sb.run(max_iter=50, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)
        T[rej] = sb.T
        mse[rej] = sb.mse
    return T, mse, {"fallback": nrej, "accepted": conv}
