"""The GoP encoder's fitting cloud over the C ABI (pvvc_fitting_clouds):
PatchFitting::Compute with direct clustering (src/patch/patch_fitting.cc:
92-381) -- an octree descent over a GoP's registered patches on the host, the
k-means of every clustering cell on the GPU."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


class Fitter:
    def __init__(self):
        self.h = L.vp()
        L.check(L.lib().pvvc_fitter_create(C.byref(self.h)), "pvvc_fitter_create")

    def close(self):
        if self.h:
            L.lib().pvvc_fitter_destroy(self.h)
            self.h = L.vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fit(self, gops, seeds=None, clustering_ths: float = 1.0, clustering_err_ths: float = 0.1, max_iter: int = 100,
            stream: int = 0):
        """gops: a list of GoPs, each a list of registered patches (float32
        [n,3], frame order).  Returns (one fitting cloud per GoP, stats)."""
        pats = [np.ascontiguousarray(p, np.float32).reshape(-1, 3) for g in gops for p in g]
        gop_patch = np.zeros(len(gops) + 1, np.int32)
        gop_patch[1:] = np.cumsum([len(g) for g in gops])
        patch_off = np.zeros(len(pats) + 1, np.uint32)
        patch_off[1:] = np.cumsum([p.shape[0] for p in pats])
        xyz = np.concatenate(pats) if pats else np.zeros((0, 3), np.float32)
        seeds = np.ascontiguousarray(np.ones(len(gops), np.uint32) if seeds is None else seeds, np.uint32)
        cap = int(patch_off[-1]) + 16
        out = np.zeros((cap, 3), np.float32)
        off = np.zeros(len(gops) + 1, np.uint64)
        st = np.zeros(4, np.int32)
        p = lambda a, t: a.ctypes.data_as(t)
        L.check(L.lib().pvvc_fitting_clouds(self.h, len(gops), p(gop_patch, L.i32p), p(patch_off, L.u32p),
                                            p(xyz, L.f32p), p(seeds, L.u32p), clustering_ths, clustering_err_ths,
                                            max_iter, p(out, L.f32p), cap, p(off, L.u64p), p(st, L.i32p), stream),
                "pvvc_fitting_clouds")
        clouds = [out[int(off[g]):int(off[g + 1])].copy() for g in range(len(gops))]
        return clouds, {"cells": int(st[0]), "iterations": int(st[1]), "empty_redraws": int(st[2]),
                        "device_rounds": int(st[3])}
