"""Seeded synthetic sequences standing in for the 8i vox10 data the reference
configs name (which are not available): see host/synth.h."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as L


def config(name: str, **over) -> L.SynthConfig:
    """Named workloads.
    'gof8'    one GoP of 8 frames, ~100k points per frame on a 512^3 grid,
              12 primitives (axes 20-120), ~64 patches of 800-2500 points, q=8.
    'seq300'  300 frames, ~800k points on a 1024^3 grid, 20 primitives
              (axes 40-240), GoP 30, ~500 patches lognormal(median 1500)
              clipped to [200, 8000], q=8 (qp overridable).
    'tiny'    a few small patches for quick checks.
    zstd_level=L (any workload): payloads zstd-compressed at level L where
    that makes them smaller, as the reference encoder does with its
    configs' zstd_level (22 in every config the reference ships)."""
    nthreads = over.pop("nthreads", os.cpu_count() or 4)
    if name == "gof8":
        c = dict(grid_bits=9, nprims=12, axis_min=20, axis_max=120, target_points=115_000, nframes=8, gof=8,
                 size_mode=0, size_a=800, size_b=2500, size_min=800, size_max=2500, qp_i=8, qp_p=8)
    elif name == "seq300":
        c = dict(grid_bits=10, nprims=20, axis_min=40, axis_max=240, target_points=920_000, nframes=300, gof=30,
                 size_mode=1, size_a=1500, size_b=0.5, size_min=200, size_max=8000, qp_i=8, qp_p=8)
    elif name == "tiny":
        c = dict(grid_bits=7, nprims=3, axis_min=10, axis_max=30, target_points=3000, nframes=4, gof=4,
                 size_mode=0, size_a=100, size_b=400, size_min=100, size_max=400, qp_i=8, qp_p=8)
    else:
        raise ValueError(name)
    c.update(dict(rot_deg=3.0, trans_vox=2.0, jitter=0.3, color_noise=4.0, seed=0, nthreads=nthreads, zstd_level=0))
    c.update(over)
    return L.SynthConfig(**c)


class Synth:
    def __init__(self, cfg: L.SynthConfig):
        h = L.vp()
        L.check(L.lib().pvvc_synth_create(C.byref(cfg), C.byref(h)), "pvvc_synth_create")
        self.h = h
        self.cfg = cfg
        self._encoded = False

    def close(self):
        if self.h:
            L.lib().pvvc_synth_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def gof_count(self) -> int:
        return int(L.lib().pvvc_synth_gof_count(self.h))

    def patch_count(self, gof: int) -> int:
        return int(L.lib().pvvc_synth_patch_count(self.h, gof))

    def patch(self, gof: int, p: int):
        """(xyz [n,3], yuv [nframes,n,3] as the encoder sees it, mv [nframes,4,4] row-major)."""
        n = C.c_uint32(0)
        nf = C.c_int32(0)
        L.check(L.lib().pvvc_synth_patch(self.h, gof, p, None, None, None, C.byref(n), C.byref(nf)), "synth_patch")
        xyz = np.zeros((n.value, 3), np.float32)
        yuv = np.zeros((nf.value, n.value, 3), np.float32)
        mv = np.zeros((nf.value, 16), np.float32)
        L.check(L.lib().pvvc_synth_patch(self.h, gof, p, xyz.ctypes.data_as(L.f32p), yuv.ctypes.data_as(L.f32p),
                                         mv.ctypes.data_as(L.f32p), None, None), "synth_patch")
        return xyz, yuv, mv.reshape(nf.value, 4, 4)

    def encode(self):
        if not self._encoded:
            L.check(L.lib().pvvc_synth_encode(self.h), "synth_encode")
            self._encoded = True

    def frame_bytes(self, t: int) -> bytes:
        self.encode()
        p = L.u8p()
        n = C.c_uint64(0)
        L.check(L.lib().pvvc_synth_frame(self.h, t, C.byref(p), C.byref(n)), "synth_frame")
        return C.string_at(p, n.value)

    def frames(self) -> list[bytes]:
        self.encode()
        return [self.frame_bytes(t) for t in range(self.cfg.nframes)]
