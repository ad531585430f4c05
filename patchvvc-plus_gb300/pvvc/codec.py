"""Python mirror of the reference's codec interface over the C ABI.

  Decoder           ~ the per-patch-index InvertRAHTOctree handlers plus
                      PVVCDecompression (src/octree/invert_raht_octree.cc,
                      src/codec/pvvc_decompression.cc): decode .frame bytes.
  Plan / decode     ~ launch_cudaProcess (src/cuda/render/CUDA2OpenGL.cu:68-74)
                      on device-resident batches.
  encode_patch_gop  ~ GoPEncoding::Encode's per-patch back end
                      (src/patch/GoP_encoding.cc:152-205).
  rlgr_encode/_decode ~ RLGREncoder / RLGRDecoder (src/common/entropy_codec.cc).
Errors raise PvvcError carrying the PVVC_* status, as the reference raises
vvc::common::Exception.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .frame import Batch


def _p(a, t):
    return a.ctypes.data_as(t)


def rlgr_encode(sym) -> bytes:
    sym = np.ascontiguousarray(sym, np.int64)
    cap = 16 * sym.size + 64
    out = np.zeros(cap, np.uint8)
    n = L.lib().pvvc_rlgr_encode(_p(sym, L.i64p), sym.size, _p(out, L.u8p), cap)
    if n < 0:
        raise L.PvvcError(int(-n), "rlgr_encode")
    return out[:n].tobytes()


def rlgr_decode(data: bytes, nsym: int) -> np.ndarray:
    buf = np.frombuffer(data, np.uint8).copy() if data else np.zeros(1, np.uint8)
    out = np.zeros(max(nsym, 1), np.int64)
    L.check(L.lib().pvvc_rlgr_decode_host(_p(buf, L.u8p), len(data), nsym, _p(out, L.i64p)), "rlgr_decode")
    return out[:nsym]


def encode_patch_gop(xyz: np.ndarray, yuv: np.ndarray, qps) -> tuple[bytes, int, list[bytes]]:
    """Geometry payload, slice size and one colour payload per frame.
    yuv: (nframes, n, 3): frame 0 absolute, later frames residuals."""
    xyz = np.ascontiguousarray(xyz, np.float32)
    yuv = np.ascontiguousarray(yuv, np.float32)
    n = xyz.shape[0]
    nf = yuv.shape[0]
    qp = np.ascontiguousarray(qps, np.uint8)
    gcap = 25 + 32 * n + 64
    ccap = 64 * n + 256
    geo = np.zeros(gcap, np.uint8)
    col = np.zeros(nf * ccap, np.uint8)
    glen = C.c_uint64(0)
    clen = np.zeros(nf, np.uint64)
    nl = C.c_uint32(0)
    L.check(L.lib().pvvc_encode_patch_gop(_p(xyz, L.f32p), n, _p(yuv, L.f32p), nf, _p(qp, L.u8p), _p(geo, L.u8p), gcap,
                                          C.byref(glen), _p(col, L.u8p), ccap, _p(clen, L.u64p), C.byref(nl)),
            "encode_patch_gop")
    cols = [col[f * ccap:f * ccap + int(clen[f])].tobytes() for f in range(nf)]
    return geo[:glen.value].tobytes(), int(nl.value), cols


class Decoder:
    """Device-resident per-patch decoder state (pvvc_state): `nslots` slots,
    each holding one patch's octree (<= max_leaves leaves, <= max_nodes
    internal nodes) and reference colours."""

    def __init__(self, nslots: int = 1024, max_leaves: int = 10000, max_nodes: int | None = None):
        if max_nodes is None:
            max_nodes = max_leaves * 2
        h = L.vp()
        L.check(L.lib().pvvc_state_create(nslots, max_leaves, max_nodes, C.byref(h)), "pvvc_state_create")
        self.h = h
        self.nslots, self.max_leaves, self.max_nodes = nslots, max_leaves, max_nodes

    def close(self):
        if self.h:
            L.lib().pvvc_state_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self, stream: int = 0):
        L.check(L.lib().pvvc_state_reset(self.h, stream), "pvvc_state_reset")

    def decode_frames(self, frames: list[bytes], stream: int = 0, out=None):
        """End-to-end host call: .frame bytes in, (xyz float32 [P,3], rgb
        uint8 [P,3], per-slice status int32) out.  out: optional (xyz, rgb)
        host arrays of at least P rows to decode into (page-locked ones are
        written by the GPU directly)."""
        nf = len(frames)
        bufs = [np.frombuffer(b, np.uint8) for b in frames]
        ptrs = (L.u8p * max(nf, 1))(*[_p(b, L.u8p) for b in bufs])
        lens = np.array([len(b) for b in frames], np.uint64)
        npts = C.c_uint64(0)
        # query the point and slice counts first
        rc = L.lib().pvvc_decode_frames_host(self.h, nf, ptrs, _p(lens, L.u64p), None, None, 0, C.byref(npts), None, 0,
                                             stream)
        if rc not in (0, 11):
            raise L.PvvcError(rc, "pvvc_decode_frames_host")
        from .frame import parse_frame
        nsl = sum(parse_frame(b).n for b in frames)
        P = int(npts.value)
        if out is not None:
            xyz, rgb = out
            if xyz.shape[0] < P or rgb.shape[0] < P or xyz.dtype != np.float32 or rgb.dtype != np.uint8:
                raise ValueError("out arrays too small or of the wrong type")
            if not (xyz.flags.c_contiguous and rgb.flags.c_contiguous):
                raise ValueError("out arrays must be contiguous")
        else:
            xyz = np.zeros((max(P, 1), 3), np.float32)
            rgb = np.zeros((max(P, 1), 3), np.uint8)
        st = np.zeros(max(nsl, 1), np.int32)
        L.check(L.lib().pvvc_decode_frames_host(self.h, nf, ptrs, _p(lens, L.u64p), _p(xyz, L.f32p), _p(rgb, L.u8p),
                                                xyz.shape[0] if out is not None else P, C.byref(npts), _p(st, L.i32p), nsl,
                                                stream), "pvvc_decode_frames_host")
        return xyz[:P], rgb[:P], st[:nsl]


def _desc(b: Batch):
    keep = [np.ascontiguousarray(x) for x in (b.slot, b.type, b.size, b.qp, b.mv, b.geo_off, b.geo_size, b.col_off,
                                              b.col_size, b.out_off)]
    k = keep
    d = L.BatchDesc(b.nslices, _p(k[0], L.i32p), _p(k[1], L.u8p), _p(k[2], L.u32p), _p(k[3], L.u8p), _p(k[4], L.f32p),
                    _p(k[5], L.u64p), _p(k[6], L.u32p), _p(k[7], L.u64p), _p(k[8], L.u32p), _p(k[9], L.u64p))
    return d, keep


def _tune(t) -> L.Tune:
    if t is None:
        return L.Tune(0, 0, 0, 0, 0, 0)
    if isinstance(t, L.Tune):
        return t
    if isinstance(t, dict):
        return L.Tune(int(t.get("group_ctas_per_sm", 0)), int(t.get("min_group", 0)), int(t.get("rlgr_block", 0)),
                      int(t.get("rlgr_long_ctas", 0)), int(t.get("rlgr_mid_pct", 0)), int(t.get("rlgr_long_lanes", 0)))
    return L.Tune(*[int(x) for x in t])


def tune_dict(t: L.Tune) -> dict:
    return {"group_ctas_per_sm": int(t.group_ctas_per_sm), "min_group": int(t.min_group), "rlgr_block": int(t.rlgr_block),
            "rlgr_long_ctas": int(t.rlgr_long_ctas), "rlgr_mid_pct": int(t.rlgr_mid_pct),
            "rlgr_long_lanes": int(t.rlgr_long_lanes)}


def autotune(b: Batch, dec: "Decoder", payload_ptr: int, reps: int = 3, stream: int = 0) -> tuple[dict, float]:
    """pvvc_plan_autotune: the fastest launch shapes for this batch and their
    median device time (ms).  Decodes the batch for real into `dec`."""
    d, keep = _desc(b)
    best = L.Tune(0, 0, 0)
    ms = C.c_float(0)
    L.check(L.lib().pvvc_plan_autotune(C.byref(d), dec.h, payload_ptr, reps, stream, C.byref(best), C.byref(ms)),
            "pvvc_plan_autotune")
    del keep
    return tune_dict(best), float(ms.value)


class Plan:
    """A device work queue for one packed Batch (pvvc_plan), with optional
    launch shapes (a pvvc_tune as dict / tuple; None = defaults)."""

    def __init__(self, b: Batch, tune=None):
        self.batch = b
        d, self._keep = _desc(b)
        h = L.vp()
        t = _tune(tune)
        L.check(L.lib().pvvc_plan_create_tuned(C.byref(d), C.byref(t), C.byref(h)), "pvvc_plan_create")
        self.h = h
        tp = C.c_uint64(0)
        wb = C.c_uint64(0)
        L.check(L.lib().pvvc_plan_query(h, C.byref(tp), C.byref(wb)), "pvvc_plan_query")
        self.total_points = int(tp.value)
        self.workspace_bytes = int(wb.value)

    def info(self) -> dict:
        i = L.PlanInfo()
        L.check(L.lib().pvvc_plan_info_get(self.h, C.byref(i)), "pvvc_plan_info_get")
        out = {k: int(getattr(i, k)) for k, _ in L.PlanInfo._fields_ if k != "tune"}
        out["tune"] = tune_dict(i.tune)
        return out

    def close(self):
        if self.h:
            L.lib().pvvc_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def decode(self, dec: Decoder, payload_ptr: int, xyz_ptr: int, rgb_ptr: int, points24_ptr: int, status_ptr: int,
               workspace_ptr: int, workspace_bytes: int, stream: int = 0) -> None:
        """pvvc_decode with raw device pointers (0 = not wanted)."""
        L.check(L.lib().pvvc_decode(self.h, dec.h, payload_ptr, xyz_ptr or None, rgb_ptr or None, points24_ptr or None,
                                    status_ptr or None, workspace_ptr, workspace_bytes, stream), "pvvc_decode")

    def graph(self, dec: Decoder, payload_ptr: int, xyz_ptr: int, rgb_ptr: int, points24_ptr: int, status_ptr: int,
              workspace_ptr: int, workspace_bytes: int) -> "Graph":
        """The decode of this plan with these buffers, captured in a CUDA graph."""
        return Graph(self, dec, payload_ptr, xyz_ptr, rgb_ptr, points24_ptr, status_ptr, workspace_ptr, workspace_bytes)


class Graph:
    """pvvc_graph: one planned decode replayed by a single graph launch."""

    def __init__(self, plan: Plan, dec: Decoder, payload_ptr, xyz_ptr, rgb_ptr, points24_ptr, status_ptr, workspace_ptr,
                 workspace_bytes):
        self._refs = (plan, dec)  # the graph bakes in their device buffers
        h = L.vp()
        L.check(L.lib().pvvc_graph_create(plan.h, dec.h, payload_ptr, xyz_ptr or None, rgb_ptr or None,
                                          points24_ptr or None, status_ptr or None, workspace_ptr, workspace_bytes,
                                          C.byref(h)), "pvvc_graph_create")
        self.h = h

    def launch(self, stream: int = 0) -> None:
        L.check(L.lib().pvvc_graph_launch(self.h, stream), "pvvc_graph_launch")

    def close(self):
        if self.h:
            L.lib().pvvc_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def patch_leaf_yuv(xyz: np.ndarray, yuv: np.ndarray) -> tuple[bytes, int, np.ndarray]:
    """Geometry payload, leaf count and per-frame leaf signal (frames x
    leaves x 3, each leaf's mean YUV in decode leaf order) of one patch.
    yuv: (nframes, n, 3): frame 0 absolute, later frames residuals."""
    xyz = np.ascontiguousarray(xyz, np.float32)
    yuv = np.ascontiguousarray(yuv, np.float32)
    n, nf = xyz.shape[0], yuv.shape[0]
    geo = np.zeros(25 + 32 * n + 64, np.uint8)
    leaf = np.zeros((nf, n, 3), np.float32)
    glen = C.c_uint64(0)
    nl = C.c_uint32(0)
    L.check(L.lib().pvvc_patch_leaf_yuv(_p(xyz, L.f32p), n, _p(yuv, L.f32p), nf, _p(geo, L.u8p), geo.size, C.byref(glen),
                                        _p(leaf, L.f32p), n, C.byref(nl)), "pvvc_patch_leaf_yuv")
    k = int(nl.value)
    return geo[:glen.value].tobytes(), k, np.ascontiguousarray(leaf[:, :k])


class Encoder:
    """GPU colour encoder (pvvc_encode_colors): forward RAHT, quantisation and
    RLGR of a batch of slices on the device."""

    def __init__(self):
        self.h = L.vp()
        L.check(L.lib().pvvc_encoder_create(C.byref(self.h)), "pvvc_encoder_create")

    def close(self):
        if self.h:
            L.lib().pvvc_encoder_destroy(self.h)
            self.h = L.vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def encode(self, batch: Batch, dec: "Decoder", payload_ptr: int, leaf_yuv_ptr: int, out_ptr: int,
               out_off: np.ndarray, out_cap: np.ndarray, out_len_ptr: int, status_ptr: int, stream: int = 0) -> None:
        """Device buffers by pointer: payload (the batch's, 16-byte aligned),
        leaf_yuv (float, slice k at 3*batch.out_off[k]), out (bytes), out_len
        (uint32 per slice), status (int32 per slice).  out_off / out_cap:
        host uint64 / uint32 arrays (multiples of 4)."""
        d, keep = _desc(batch)
        off = np.ascontiguousarray(out_off, np.uint64)
        cap = np.ascontiguousarray(out_cap, np.uint32)
        L.check(L.lib().pvvc_encode_colors(self.h, C.byref(d), dec.h, payload_ptr, leaf_yuv_ptr, out_ptr,
                                           _p(off, L.u64p), _p(cap, L.u32p), out_len_ptr, status_ptr, stream),
                "pvvc_encode_colors")
