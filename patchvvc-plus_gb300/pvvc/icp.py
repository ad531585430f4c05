"""Batched ICP over the C ABI (pvvc_icp_batch / pvvc_cloud_mse_batch) and the
seeded patch-pair workload that stands in for the encoder's registration
calls (PatchFitting::AddPatch, src/patch/patch_fitting.cc:58-79;
PatchesRegistration::Task, src/registration/patches_registration.cc:80-90).

Device buffers are torch tensors (plumbing only); the work runs in
libpvvc_gb300.so."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L


def rotation(axis, deg) -> np.ndarray:
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    th = np.deg2rad(deg)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * (K @ K)


@dataclass
class Pairs:
    src: list          # float32 [n,3] per pair (int32 10-bit coordinates as floats)
    tgt: list          # float32 [m,3] per pair
    T_true: np.ndarray  # [npairs,4,4]: maps src onto the clean target

    @property
    def n(self) -> int:
        return len(self.src)


def make_pairs(npairs: int, seed: int = 0, max_deg: float = 15.0, max_trans: float = 20.0, noise: float = 0.5,
               outliers: float = 0.05, synth=None) -> Pairs:
    """Each source is a patch of the seeded synthetic surface (lognormal sizes,
    median 1500, clipped to [200, 8000], 10-bit integer coordinates); its
    target is the source rotated by U(0, max_deg) degrees about a uniform axis
    through its centroid, translated by U(-max_trans, max_trans)^3, with
    N(0, noise) jitter and `outliers` x n extra points uniform in its box."""
    from .synth import Synth, config
    if synth is None:
        synth = Synth(config("seq300", nframes=1, gof=1, seed=seed))
    npat = synth.patch_count(0)
    rng = np.random.default_rng(seed + 12345)
    src, tgt, Ts = [], [], []
    cache = {}
    for i in range(npairs):
        p = int(rng.integers(0, npat))
        if p not in cache:
            cache[p] = synth.patch(0, p)[0]
        s = cache[p]
        c = s.mean(0)
        R = rotation(rng.normal(size=3), rng.uniform(0, max_deg))
        t = rng.uniform(-max_trans, max_trans, 3)
        T = np.eye(4)
        T[:3, :3] = R
        T[:3, 3] = c + t - R @ c
        q = (s.astype(np.float64) - c) @ R.T + c + t + rng.normal(0, noise, s.shape)
        k = int(round(outliers * s.shape[0]))
        lo, hi = q.min(0), q.max(0)
        q = np.concatenate([q, rng.uniform(lo, hi, (k, 3))])
        src.append(s.astype(np.float32))
        tgt.append(q.astype(np.float32))
        Ts.append(T)
    return Pairs(src, tgt, np.array(Ts))


def make_pairs_packed(npairs: int, seed: int = 0, max_deg: float = 15.0, max_trans: float = 20.0, noise: float = 0.5,
                      outliers: float = 0.05, synth=None, device="cuda"):
    """The make_pairs workload generated in one vectorised pass on `device`
    (torch ops; for large training sets).  Returns packed device clouds
    (src [S,3] f32, src_off [n+1] i32, tgt [T,3] f32, tgt_off [n+1] i32)
    and T_true [n,4,4] (numpy float64)."""
    import torch
    from .synth import Synth, config
    if synth is None:
        synth = Synth(config("seq300", nframes=1, gof=1, seed=seed))
    npat = synth.patch_count(0)
    pats = [synth.patch(0, p)[0].astype(np.float32) for p in range(npat)]
    dev = torch.device(device)
    g = torch.Generator(device=dev).manual_seed(seed + 54321)
    f64 = torch.float64
    sizes = torch.tensor([p.shape[0] for p in pats], device=dev)
    poff = torch.cat([torch.zeros(1, dtype=torch.int64, device=dev), torch.cumsum(sizes, 0)])
    allp = torch.from_numpy(np.concatenate(pats)).to(dev, f64)
    cent = torch.stack([torch.from_numpy(p.astype(np.float64).mean(0)) for p in pats]).to(dev)
    pid = torch.randint(0, npat, (npairs,), generator=g, device=dev)
    ax = torch.randn(npairs, 3, generator=g, device=dev, dtype=f64)
    ax = ax / ax.norm(dim=1, keepdim=True)
    th = torch.deg2rad(torch.rand(npairs, generator=g, device=dev, dtype=f64) * max_deg)
    K = torch.zeros(npairs, 3, 3, device=dev, dtype=f64)
    K[:, 0, 1], K[:, 0, 2], K[:, 1, 2] = -ax[:, 2], ax[:, 1], -ax[:, 0]
    K[:, 1, 0], K[:, 2, 0], K[:, 2, 1] = ax[:, 2], -ax[:, 1], ax[:, 0]
    R = torch.eye(3, device=dev, dtype=f64) + torch.sin(th)[:, None, None] * K + (1 - torch.cos(th))[:, None, None] * (K @ K)
    t = (torch.rand(npairs, 3, generator=g, device=dev, dtype=f64) * 2 - 1) * max_trans
    n = sizes[pid]
    soff = torch.cat([torch.zeros(1, dtype=torch.int64, device=dev), torch.cumsum(n, 0)])
    owner = torch.repeat_interleave(torch.arange(npairs, device=dev), n)
    local = torch.arange(int(soff[-1]), device=dev) - soff[:-1][owner]
    S = allp[poff[pid][owner] + local]
    c = cent[pid]
    Q = torch.bmm(R[owner], (S - c[owner]).unsqueeze(2)).squeeze(2) + (c + t)[owner]
    Q = Q + torch.randn(Q.shape, generator=g, device=dev, dtype=f64) * noise
    lo = torch.full((npairs, 3), float("inf"), device=dev, dtype=f64).scatter_reduce(0, owner[:, None].expand(-1, 3), Q, "amin")
    hi = torch.full((npairs, 3), float("-inf"), device=dev, dtype=f64).scatter_reduce(0, owner[:, None].expand(-1, 3), Q, "amax")
    k = torch.round(outliers * n.to(f64)).to(torch.int64)
    oown = torch.repeat_interleave(torch.arange(npairs, device=dev), k)
    O = lo[oown] + torch.rand(int(k.sum()), 3, generator=g, device=dev, dtype=f64) * (hi - lo)[oown]
    toff = torch.cat([torch.zeros(1, dtype=torch.int64, device=dev), torch.cumsum(n + k, 0)])
    tgt = torch.empty(int(toff[-1]), 3, device=dev, dtype=torch.float32)
    tgt[toff[:-1][owner] + local] = Q.float()                      # the moved source first, then its outliers
    kof = torch.cat([torch.zeros(1, dtype=torch.int64, device=dev), torch.cumsum(k, 0)])
    ko = torch.arange(int(k.sum()), device=dev) - kof[:-1][oown]
    tgt[toff[:-1][oown] + n[oown] + ko] = O.float()
    T = torch.eye(4, device=dev, dtype=f64).repeat(npairs, 1, 1)
    T[:, :3, :3] = R
    T[:, :3, 3] = c + t - torch.bmm(R, c.unsqueeze(2)).squeeze(2)
    return S.float(), soff.to(torch.int32), tgt, toff.to(torch.int32), T.cpu().numpy()


def _pack(clouds):
    off = np.zeros(len(clouds) + 1, np.uint32)
    off[1:] = np.cumsum([c.shape[0] for c in clouds])
    return np.concatenate(clouds).astype(np.float32), off


class IcpBatch:
    """Device-resident batch of (source, target) pairs."""

    def __init__(self, pairs: Pairs | None, device="cuda", packed=None):
        """pairs: host clouds, or packed=(src, src_off, tgt, tgt_off) device
        tensors as make_pairs_packed returns them."""
        import torch
        self.torch = torch
        dev = torch.device(device)
        if packed is None:
            s, so = _pack(pairs.src)
            t, to = _pack(pairs.tgt)
            self.src = torch.from_numpy(s).to(dev)
            self.tgt = torch.from_numpy(t).to(dev)
            self.soff = torch.from_numpy(so.astype(np.int32)).to(dev)
            self.toff = torch.from_numpy(to.astype(np.int32)).to(dev)
        else:
            self.src, self.soff, self.tgt, self.toff = packed
        self.n = int(self.soff.numel()) - 1
        self.ns, self.nt = int(self.src.shape[0]), int(self.tgt.shape[0])
        b = C.c_uint64(0)
        L.check(L.lib().pvvc_icp_workspace_size(self.n, self.ns, self.nt, C.byref(b)), "pvvc_icp_workspace_size")
        self.ws = torch.empty(max(int(b.value), 256), dtype=torch.uint8, device=dev)
        self.T = torch.empty((self.n, 16), dtype=torch.float32, device=dev)
        self.mse = torch.empty(self.n, dtype=torch.float32, device=dev)
        self.iters = torch.empty(self.n, dtype=torch.int32, device=dev)
        self.conv = torch.empty(self.n, dtype=torch.uint8, device=dev)
        self.dev = dev

    def run(self, init=None, max_corr_dist=1e6, max_iter=50, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6,
            stream=None):
        """Launch pvvc_icp_batch (stream-ordered, no sync).  init: device
        tensor [n,16] row-major or None."""
        prm = L.IcpParams(max_corr_dist, max_iter, fitness_eps, transform_eps, mse_abs_eps)
        sp = stream if stream is not None else self.torch.cuda.current_stream(self.dev).cuda_stream
        L.check(L.lib().pvvc_icp_batch(self.n, self.src.data_ptr(), self.soff.data_ptr(), self.tgt.data_ptr(),
                                       self.toff.data_ptr(), None if init is None else init.data_ptr(), C.byref(prm),
                                       self.T.data_ptr(), self.mse.data_ptr(), self.iters.data_ptr(), self.conv.data_ptr(),
                                       self.ws.data_ptr(), self.ws.numel(), self.ns, self.nt, sp), "pvvc_icp_batch")

    def results(self):
        self.torch.cuda.synchronize(self.dev)
        return (self.T.cpu().numpy().reshape(-1, 4, 4), self.mse.cpu().numpy(), self.iters.cpu().numpy(),
                self.conv.cpu().numpy().astype(bool))

    def cloud_mse(self, T=None, stream=None):
        """ICPBase::CloudMSE of every pair after transforming the source by T
        (device [n,16], default: the last ICP result)."""
        T = self.T if T is None else T
        out = self.torch.empty(self.n, dtype=self.torch.float32, device=self.dev)
        sp = stream if stream is not None else self.torch.cuda.current_stream(self.dev).cuda_stream
        L.check(L.lib().pvvc_cloud_mse_batch(self.n, self.src.data_ptr(), self.soff.data_ptr(), self.tgt.data_ptr(),
                                             self.toff.data_ptr(), T.data_ptr(), out.data_ptr(), self.ws.data_ptr(),
                                             self.ws.numel(), self.ns, self.nt, sp), "pvvc_cloud_mse_batch")
        self.torch.cuda.synchronize(self.dev)
        return out.cpu().numpy()


class KnnColorBatch:
    """Device-resident colour interpolation of the GoP encoder
    (pvvc_knn_colors_batch; GoPEncoding::Interpolation and its k-NN loop,
    src/patch/GoP_encoding.cc:73-95,131-150).  queries: float32 [n,3] clouds
    (a pair names one by query_of[p]); sources: float32 [m,3] patches with
    rgbs: uint8 [m,3]; base: optional base pair per pair (-1: none), which
    turns a pair into the residual against its base."""

    def __init__(self, queries, query_of, sources, rgbs, k=10, base=None, device="cuda"):
        import torch
        self.torch = torch
        dev = torch.device(device)
        self.n = len(sources)
        q = np.ascontiguousarray(np.concatenate(queries) if queries else np.zeros((0, 3)), np.float32)
        qstart = np.zeros(len(queries) + 1, np.uint64)
        qstart[1:] = np.cumsum([x.shape[0] for x in queries])
        qof = np.asarray(query_of, np.int64)
        self.qn = np.array([queries[i].shape[0] for i in qof], np.uint32)
        qoff = qstart[qof].astype(np.uint64)
        self.out_off = np.zeros(self.n, np.uint64)
        self.out_off[1:] = np.cumsum(self.qn.astype(np.uint64))[:-1]
        s, so = _pack(sources)
        c = np.ascontiguousarray(np.concatenate(rgbs), np.uint8)
        self.ns = int(s.shape[0])
        self.k = int(k)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        self.q, self.qoff, self.qn_d = t(q), t(qoff.view(np.int64)), t(self.qn.view(np.int32))
        self.src, self.rgb, self.soff = t(s), t(c), t(so.view(np.int32))
        self.base = None if base is None else t(np.asarray(base, np.int32))
        self.out_off_d = t(self.out_off.view(np.int64))
        self.total = int(self.qn.sum())
        self.yuv = torch.empty((max(self.total, 1), 3), dtype=torch.float32, device=dev)
        self.status = torch.empty(max(self.n, 1), dtype=torch.int32, device=dev)
        b = C.c_uint64(0)
        L.check(L.lib().pvvc_knn_colors_workspace_size(self.n, self.ns, C.byref(b)), "pvvc_knn_colors_workspace_size")
        self.ws = torch.empty(max(int(b.value), 256), dtype=torch.uint8, device=dev)
        self.dev = dev

    def run(self, stream=None):
        """Launch pvvc_knn_colors_batch (stream-ordered, no sync)."""
        sp = stream if stream is not None else self.torch.cuda.current_stream(self.dev).cuda_stream
        L.check(L.lib().pvvc_knn_colors_batch(self.n, self.q.data_ptr(), self.qoff.data_ptr(), self.qn_d.data_ptr(),
                                              self.src.data_ptr(), self.rgb.data_ptr(), self.soff.data_ptr(), self.k,
                                              None if self.base is None else self.base.data_ptr(), self.yuv.data_ptr(),
                                              self.out_off_d.data_ptr(), self.status.data_ptr(), self.ws.data_ptr(),
                                              self.ws.numel(), self.ns, sp), "pvvc_knn_colors_batch")

    def results(self):
        """Per pair its YUV [n,3] (numpy) and the status array."""
        self.torch.cuda.synchronize(self.dev)
        y = self.yuv.cpu().numpy()
        return [y[int(a):int(a) + int(m)] for a, m in zip(self.out_off, self.qn)], self.status.cpu().numpy()[:self.n]


def rotation_error_deg(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """Angle of A[:3,:3] B[:3,:3]^T per pair, degrees."""
    R = np.einsum("nij,nkj->nik", A[:, :3, :3].astype(np.float64), B[:, :3, :3].astype(np.float64))
    c = np.clip((np.trace(R, axis1=1, axis2=2) - 1) / 2, -1, 1)
    return np.rad2deg(np.arccos(c))
