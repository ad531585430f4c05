"""The GoP encode flow with registration, end to end on the GPU, and the
decoded sequence's PSNR.

Restates the reference encoder's per-GoP steps:
  PatchFitting::AddPatch (src/patch/patch_fitting.cc:34-90)
      each frame's patch is registered by ICP onto the GoP's fitting cloud
      (here the patch of the GoP's first frame); the registration is accepted
      when ICPBase::CloudMSE <= fitting_ths, and its motion mv = T * mv;
  GoPEncoding::Encode (src/patch/GoP_encoding.cc:120-205)
      Slice.mv = inverse(Patch.mv); every frame's colours are interpolated
      onto the fitting cloud (k nearest points of the registered patch),
      later frames as residuals against frame 0; RAHT, quantisation, RLGR;
then decodes the bitstream (pvvc_decode_frames_host) and measures each
decoded frame against its source frame with common::MSE::Compute
(registration_base.cc:160-223) and the decoder's PSNR
(pvvc_decompression.cc:151-171).

The source frames stand in for the voxelised captures the reference reads:
every patch of the synthetic sequence (its GoP geometry and per-frame
colours) moved by the frame's rigid motion, jittered N(0, jitter) and rounded
to the voxel grid, duplicates dropped.  The registration is pluggable, so the
same flow measures plain ICP from the identity, the learned initial guess,
and the generator's true motion.

GPU work: pvvc_icp_batch (or the learned registration), pvvc_cloud_mse_batch,
pvvc_knn_colors_batch, pvvc_encode_colors, pvvc_decode_frames_host,
pvvc_cloud_quality.  The host only moves points into batches."""
from __future__ import annotations

import time

import numpy as np

from .frame import Frame, pack_frames, write_frame
from .icp import IcpBatch, KnnColorBatch, Pairs
from .quality import Quality, psnr


def yuv_to_rgb(yuv: np.ndarray) -> np.ndarray:
    """ColorYUV::ConvertRGB (include/common/common.h:154-158), float32 ops,
    rounded half away from zero and clamped."""
    f = np.float32
    y, u, v = yuv[:, 0].astype(f), yuv[:, 1].astype(f), yuv[:, 2].astype(f)
    rgb = np.stack([y + f(1.402) * (v - f(128)), (y - f(0.3441) * (u - f(128))) - f(0.7141) * (v - f(128)),
                    y + f(1.772) * (u - f(128))], 1).astype(np.float64)
    return np.clip(np.sign(rgb) * np.floor(np.abs(rgb) + 0.5), 0, 255).astype(np.uint8)


class GopSource:
    """The source frames of one GoP of a synthetic sequence, per patch: the
    fitting cloud (the GoP geometry at its first frame), the per-frame
    source patches (moved, jittered, voxelised) with RGB, and the true
    per-frame motion."""

    def __init__(self, synth, gof_index: int, jitter: float = 0.3, seed: int = 0, nthreads: int = 16):
        import concurrent.futures as cf
        self.npatch = synth.patch_count(gof_index)
        rng0 = np.random.default_rng(seed)
        seeds = rng0.integers(0, 2**63, self.npatch)

        def one(p):
            xyz, yuv, mv = synth.patch(gof_index, p)
            rng = np.random.default_rng(int(seeds[p]))
            nf = yuv.shape[0]
            frames = []
            for f in range(nf):
                col = yuv[0] if f == 0 else yuv[0] + yuv[f]
                rgb = yuv_to_rgb(col)
                if f == 0:
                    frames.append((xyz.astype(np.float32), rgb))
                    continue
                m = mv[f].astype(np.float64)
                moved = xyz.astype(np.float64) @ m[:3, :3].T + m[:3, 3] + rng.normal(0, jitter, xyz.shape)
                vox = np.round(moved).astype(np.int64)
                key = (vox[:, 0] << 42) | ((vox[:, 1] & 0x1FFFFF) << 21) | (vox[:, 2] & 0x1FFFFF)
                _, first = np.unique(key, return_index=True)
                first.sort()
                frames.append((vox[first].astype(np.float32), rgb[first]))
            return xyz.astype(np.float32), frames, mv.astype(np.float32)

        with cf.ThreadPoolExecutor(max_workers=nthreads) as ex:
            parts = list(ex.map(one, range(self.npatch)))
        self.fit = [p[0] for p in parts]                  # fitting clouds
        self.frames = [p[1] for p in parts]               # [patch][frame] -> (xyz, rgb)
        self.true_mv = [p[2] for p in parts]              # [patch] -> [nf, 4, 4]
        self.nframes = len(self.frames[0]) if parts else 0

    def frame_cloud(self, f: int):
        """The whole source frame f: every patch's source points and RGB."""
        xs = [self.frames[p][f][0] for p in range(self.npatch)]
        cs = [self.frames[p][f][1] for p in range(self.npatch)]
        return np.concatenate(xs), np.concatenate(cs)


def register_plain(batch: IcpBatch, **kw):
    """Plain ICP from the identity (the encoder's default registration)."""
    batch.run(max_corr_dist=1e6, max_iter=kw.get("max_iter", 50), fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)
    return batch.T.clone()


def encode_decode_gop(src: GopSource, register, qp: int = 8, k: int = 10, fitting_ths: float | None = None,
                      dec=None, quality: Quality | None = None, keep_frames: bool = False) -> dict:
    """Registers every later frame's patches onto the fitting clouds with
    `register(IcpBatch) -> device T [n,16]` (source = the frame's patch
    pre-aligned by its previous frame's motion, target = the fitting cloud;
    None: the true motion), interpolates the
    colours, encodes, decodes through pvvc_decode_frames_host and measures
    each frame against its source.  Returns per-frame PSNR and the timings."""
    import torch

    from . import codec
    nf, npat = src.nframes, src.npatch
    t = {}
    # ---- registration (PatchFitting::AddPatch) ----
    # Frame by frame: each patch, pre-aligned by its previous frame's motion
    # (the reference pre-registers a frame's patches against the previous
    # frame's before fitting, patches_registration.cc:80-90), registered onto
    # the fitting cloud; T(f) = T_reg * T(f-1) maps frame f onto the fitting
    # cloud.
    t0 = time.perf_counter()
    T = np.tile(np.eye(4, dtype=np.float64), (npat, nf, 1, 1))
    gate, cms, reg_ms = [], [], 0.0
    if register is None:
        for p in range(npat):  # the true motion maps the fitting cloud onto frame f; its inverse, frame f onto it
            for f in range(1, nf):
                T[p, f] = np.linalg.inv(src.true_mv[p][f].astype(np.float64))
    else:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for f in range(1, nf):
            pre = [(src.frames[p][f][0].astype(np.float64) @ T[p, f - 1][:3, :3].T + T[p, f - 1][:3, 3]).astype(np.float32)
                   for p in range(npat)]
            b = IcpBatch(Pairs(pre, src.fit, np.zeros((npat, 4, 4))))
            torch.cuda.synchronize()
            e0.record()
            Td = register(b)
            e1.record()
            torch.cuda.synchronize()
            reg_ms += e0.elapsed_time(e1)
            Tr = Td.cpu().numpy().reshape(-1, 4, 4).astype(np.float64)
            cm = b.cloud_mse(Td)
            cms.append(cm)
            if fitting_ths is not None:
                gate.append(cm <= fitting_ths)
            for p in range(npat):
                T[p, f] = Tr[p] @ T[p, f - 1]
        cms = np.concatenate(cms)
        t["cloud_mse_mean"] = float(cms.mean())
    t["register_ms"] = reg_ms
    t["register_host_s"] = time.perf_counter() - t0
    gate = float(np.concatenate(gate).mean()) if gate else None
    pairs_n = npat * (nf - 1)
    # ---- colour interpolation onto the fitting clouds (GoPEncoding::Encode) ----
    t0 = time.perf_counter()
    queries, query_of, sources, rgbs, base = src.fit, [], [], [], []
    for p in range(npat):
        first = len(sources)
        for f in range(nf):
            x, c = src.frames[p][f]
            m = T[p, f].astype(np.float64)
            sources.append((x.astype(np.float64) @ m[:3, :3].T + m[:3, 3]).astype(np.float32) if f else x)
            rgbs.append(c)
            query_of.append(p)
            base.append(-1 if f == 0 else first)
    kb = KnnColorBatch(queries, query_of, sources, rgbs, k=k, base=base)
    kb.run()
    yuv, st = kb.results()
    assert (st == 0).all(), np.unique(st)
    # ---- RAHT + quantisation + RLGR of every slice (GPU encoder back end) ----
    geos, leaves = [], []
    for p in range(npat):
        g, nl, leaf = codec.patch_leaf_yuv(src.fit[p], np.stack(yuv[p * nf:(p + 1) * nf]))
        geos.append((g, nl))
        leaves.append(leaf)
    flist = []
    for f in range(nf):
        mv = np.stack([np.linalg.inv(T[p, f].astype(np.float64)).astype(np.float32).reshape(16) for p in range(npat)])
        flist.append(Frame(f, np.arange(npat, dtype=np.int32), np.full(npat, 1 if f == 0 else 3, np.uint8),
                           np.array([q[1] for q in geos], np.uint32), np.full(npat, qp, np.uint8), mv,
                           [q[0] if f == 0 else b"" for q in geos], [b""] * npat))
    batch = pack_frames(flist)
    leaf_yuv = np.zeros((batch.points, 3), np.float32)
    for kk in range(batch.nslices):
        f, p = kk // npat, kk % npat
        o = int(batch.out_off[kk])
        leaf_yuv[o:o + leaves[p].shape[1]] = leaves[p][f]
    enc = codec.Encoder()
    ed = codec.Decoder(nslots=npat, max_leaves=8192, max_nodes=16384)
    cap = ((8 * batch.size.astype(np.uint64) + 64 + 3) // 4 * 4).astype(np.uint32)
    off = np.concatenate([[0], np.cumsum(cap.astype(np.uint64))[:-1]]).astype(np.uint64)
    dev = torch.device("cuda")
    pay = torch.from_numpy(batch.payload).to(dev)
    ly = torch.from_numpy(leaf_yuv).to(dev)
    out = torch.zeros(int(cap.astype(np.uint64).sum()) + 16, dtype=torch.uint8, device=dev)
    olen = torch.zeros(batch.nslices, dtype=torch.int32, device=dev)
    est = torch.zeros(batch.nslices, dtype=torch.int32, device=dev)
    enc.encode(batch, ed, pay.data_ptr(), ly.data_ptr(), out.data_ptr(), off, cap, olen.data_ptr(), est.data_ptr(),
               torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert (est.cpu().numpy() == 0).all()
    ob, ol = out.cpu().numpy(), olen.cpu().numpy()
    frames_bytes, bits = [], 0
    for f in range(nf):
        cols = [ob[int(off[f * npat + p]):int(off[f * npat + p]) + int(ol[f * npat + p])].tobytes() for p in range(npat)]
        bits += 8 * sum(len(c) for c in cols) + 8 * sum(len(g) for g in flist[f].geometry)
        fr = flist[f]
        frames_bytes.append(write_frame(Frame(fr.timestamp, fr.index, fr.type, fr.size, fr.qp, fr.mv, fr.geometry, cols)))
    t["encode_host_s"] = time.perf_counter() - t0
    # ---- decode and measure ----
    t0 = time.perf_counter()
    dec = dec or codec.Decoder(nslots=npat, max_leaves=8192, max_nodes=16384)
    xyz, rgb, dst = dec.decode_frames(frames_bytes)
    assert (dst == 0).all()
    quality = quality or Quality()
    per = []
    o = 0
    for f in range(nf):
        n = sum(int(q[1]) for q in geos)
        sx, sc = src.frame_cloud(f)
        m = quality.mse(sx, sc, xyz[o:o + n], rgb[o:o + n])
        per.append(psnr(m))
        o += n
    t["decode_measure_s"] = time.perf_counter() - t0
    return {"frames": nf, "patches": npat, "pairs": pairs_n, "bits": bits, "points": int(batch.points),
            "bits_per_point": bits / max(batch.points, 1),
            "psnr_geo": float(np.mean([x["geo"] for x in per])), "psnr_y": float(np.mean([x["y"] for x in per])),
            "psnr_geo_per_frame": [round(x["geo"], 3) for x in per], "psnr_y_per_frame": [round(x["y"], 3) for x in per],
            "fitting_gate_pass": gate, "times": t, **({"frame_bytes": frames_bytes} if keep_frames else {})}
