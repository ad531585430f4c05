"""ctypes bindings for the test oracle (oracle/_build/libpvvc_oracle.so) and,
where it was built, the reference's own sources (oracle/_ref/libpvvc_ref.so).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py -- never by the shipped package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ORACLE_SO = os.path.join(_HERE, "_build", "libpvvc_oracle.so")
_REF_SO = os.path.join(_HERE, "_ref", "libpvvc_ref.so")
# the reference project's checkout (read-only); PVVC_REFERENCE_ROOT overrides
REFERENCE_ROOT = os.environ.get("PVVC_REFERENCE_ROOT", "/root/reference")

_u8p = C.POINTER(C.c_uint8)
_f32p = C.POINTER(C.c_float)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)
_u32p = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)


def build_oracle(force: bool = False) -> str:
    """Compile the C restatement with make (quick, a few seconds)."""
    if force or not os.path.exists(_ORACLE_SO) or _stale(_ORACLE_SO, ["pvvc_oracle.c", "pvvc_oracle_icp.c", "pvvc_oracle.h"]):
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "all"], check=True)
    return _ORACLE_SO


def build_reference() -> str | None:
    """Compile the reference's own sources against the shims, if the reference
    tree is present on this machine.  Returns the .so path or None."""
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "src")):
        return _REF_SO if os.path.exists(_REF_SO) else None
    # make rebuilds only when a source or a shim changed
    r = subprocess.run(["make", "-s", "-C", _HERE, "ref", f"REF={REFERENCE_ROOT}"], capture_output=True, text=True)
    return _REF_SO if r.returncode == 0 and os.path.exists(_REF_SO) else None


def _stale(target, srcs):
    t = os.path.getmtime(target)
    return any(os.path.getmtime(os.path.join(_HERE, s)) > t for s in srcs)


def _ptr(a, typ):
    return a.ctypes.data_as(typ)


class _PvoFrame(C.Structure):
    _fields_ = [
        ("n", C.c_uint32),
        ("index", _i32p),
        ("type", _u8p),
        ("size", _u32p),
        ("qp", _u8p),
        ("mv", _f32p),
        ("geo", C.POINTER(_u8p)),
        ("gsz", _u32p),
        ("col", C.POINTER(_u8p)),
        ("csz", _u32p),
        ("out_off", _u64p),
    ]


class _IcpParams(C.Structure):
    _fields_ = [("max_corr_dist", C.c_float), ("max_iter", C.c_int), ("fitness_eps", C.c_float), ("transform_eps", C.c_float),
                ("mse_abs_eps", C.c_float)]


class Oracle:
    """The C restatement of the reference codec path."""

    def __init__(self):
        lib = C.CDLL(build_oracle())
        self.lib = lib
        lib.pvo_rlgr_encode.restype = C.c_size_t
        lib.pvo_rlgr_encode.argtypes = [_i64p, C.c_size_t, _u8p, C.c_size_t]
        lib.pvo_rlgr_decode.restype = C.c_int
        lib.pvo_rlgr_decode.argtypes = [_u8p, C.c_size_t, C.c_size_t, _i64p]
        lib.pvo_encoder_new.restype = C.c_void_p
        lib.pvo_encoder_new.argtypes = [_f32p, C.c_size_t, C.c_float, C.POINTER(C.c_int)]
        lib.pvo_encoder_free.argtypes = [C.c_void_p]
        lib.pvo_encoder_leaf_count.restype = C.c_size_t
        lib.pvo_encoder_leaf_count.argtypes = [C.c_void_p]
        lib.pvo_encoder_height.restype = C.c_int
        lib.pvo_encoder_height.argtypes = [C.c_void_p]
        lib.pvo_encoder_geometry.restype = C.c_size_t
        lib.pvo_encoder_geometry.argtypes = [C.c_void_p, _u8p, C.c_size_t]
        lib.pvo_encoder_raht.restype = C.c_int
        lib.pvo_encoder_raht.argtypes = [C.c_void_p, _f32p, _f32p]
        lib.pvo_encode_colors.restype = C.c_size_t
        lib.pvo_encode_colors.argtypes = [_f32p, C.c_size_t, C.c_uint8, _u8p, C.c_size_t]
        lib.pvo_decoder_new.restype = C.c_void_p
        lib.pvo_decoder_free.argtypes = [C.c_void_p]
        lib.pvo_decoder_set_slice.restype = C.c_int
        lib.pvo_decoder_set_slice.argtypes = [C.c_void_p, C.c_uint8, C.c_uint32, C.c_uint8, _u8p, C.c_size_t, _u8p, C.c_size_t]
        lib.pvo_decoder_size.restype = C.c_size_t
        lib.pvo_decoder_size.argtypes = [C.c_void_p]
        lib.pvo_decoder_get_patch.restype = C.c_int
        lib.pvo_decoder_get_patch.argtypes = [C.c_void_p, _f32p, _f32p, _u8p]
        lib.pvo_decoder_enable_fp64.argtypes = [C.c_void_p, C.c_int]
        lib.pvo_decoder_get_yuv_fp64.restype = C.c_int
        lib.pvo_decoder_get_yuv_fp64.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        lib.pvo_transform.argtypes = [_f32p, _f32p, C.c_size_t, _f32p]
        lib.pvo_decode_frame.restype = C.c_int
        lib.pvo_decode_frame.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.POINTER(_PvoFrame), _f32p, _u8p, _i32p, C.c_int]
        if hasattr(lib, "pvo_icp_align"):
            lib.pvo_icp_align.restype = C.c_int
            lib.pvo_icp_align.argtypes = [_f32p, C.c_size_t, _f32p, C.c_size_t, _f32p, C.POINTER(_IcpParams), _f32p, _f32p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
            lib.pvo_icp_batch.restype = C.c_int
            lib.pvo_icp_batch.argtypes = [C.c_int, _f32p, _u32p, _f32p, _u32p, C.POINTER(_IcpParams), _f32p, _f32p,
                                          C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int]
            lib.pvo_cloud_mse.restype = C.c_float
            lib.pvo_cloud_mse.argtypes = [_f32p, C.c_size_t, _f32p, C.c_size_t]
            lib.pvo_fitting_cloud.restype = C.c_long
            lib.pvo_fitting_cloud.argtypes = [C.c_int, C.POINTER(_f32p), _u32p, C.c_float, C.c_float, C.c_int, C.c_uint,
                                              _f32p, C.c_size_t, C.POINTER(C.c_long)]
            lib.pvo_cloud_quality.restype = C.c_int
            lib.pvo_cloud_quality.argtypes = [_f32p, _u8p, C.c_size_t, _f32p, _u8p, C.c_size_t, C.c_int,
                                              C.POINTER(C.c_double)]
            lib.pvo_knn_colors.restype = C.c_int
            lib.pvo_knn_colors.argtypes = [_f32p, C.c_size_t, _f32p, _u8p, C.c_size_t, C.c_int, C.c_int, _f32p]
            lib.pvo_knn_colors_batch.restype = C.c_int
            lib.pvo_knn_colors_batch.argtypes = [C.c_int, _f32p, C.POINTER(C.c_uint64), _u32p, _f32p, _u8p, _u32p,
                                                 C.c_int, _f32p, C.POINTER(C.c_uint64), C.c_int]

    # ---- zstd (libzstd, the reference's dependency) ----
    def libzstd_inflate_batch(self, payloads: list, caps: list, nthreads: int):
        """ZSTD_decompress of every payload on nthreads host threads
        (ZstdDecoder::Decode, src/common/entropy_codec.cc:341-360).
        Returns (outputs, statuses, seconds of the batch call)."""
        import time
        lib = self.lib
        lib.pvo_libzstd_inflate_batch.restype = C.c_int
        n = len(payloads)
        src = np.frombuffer(b"".join(payloads) + b"\0", np.uint8).copy()
        sl = np.array([len(p) for p in payloads], np.uint32)
        so = np.zeros(n, np.uint64)
        so[1:] = np.cumsum(sl[:-1].astype(np.uint64))
        cp = np.array(caps, np.uint32)
        do = np.zeros(n, np.uint64)
        do[1:] = np.cumsum(cp[:-1].astype(np.uint64))
        dst = np.zeros(int(cp.astype(np.uint64).sum()) + 1, np.uint8)
        st = np.zeros(max(n, 1), np.int32)
        t = time.perf_counter()
        rc = lib.pvo_libzstd_inflate_batch(n, _ptr(src, _u8p), so.ctypes.data_as(C.c_void_p), sl.ctypes.data_as(C.c_void_p),
                                           _ptr(dst, _u8p), do.ctypes.data_as(C.c_void_p), cp.ctypes.data_as(C.c_void_p),
                                           _ptr(st, _i32p), nthreads)
        dt = time.perf_counter() - t
        if rc:
            raise RuntimeError("libzstd is not available")
        outs = [dst[int(do[j]):int(do[j]) + int(cp[j])].tobytes() for j in range(n)]
        return outs, st[:n].tolist(), dt

    # ---- RLGR ----
    def rlgr_encode(self, sym: np.ndarray) -> bytes:
        sym = np.ascontiguousarray(sym, dtype=np.int64)
        cap = 16 * sym.size + 64
        out = np.zeros(cap, np.uint8)
        n = self.lib.pvo_rlgr_encode(_ptr(sym, _i64p), sym.size, _ptr(out, _u8p), cap)
        if n == 0 and sym.size:
            raise RuntimeError("rlgr encode overflow")
        return out[:n].tobytes()

    def rlgr_decode(self, data: bytes, nsym: int) -> np.ndarray:
        buf = np.frombuffer(data, np.uint8).copy() if data else np.zeros(1, np.uint8)
        out = np.zeros(max(nsym, 1), np.int64)
        st = self.lib.pvo_rlgr_decode(_ptr(buf, _u8p), len(data), nsym, _ptr(out, _i64p))
        if st != 0:
            raise ValueError(f"rlgr decode status {st}")
        return out[:nsym]

    # ---- encoder ----
    def encode_patch(self, xyz: np.ndarray, yuv_frames: list[np.ndarray], qps: list[int]):
        """Geometry bytes, leaf count, and one colour payload per frame.
        yuv_frames[f] is (n,3) per input point; frame 0 is the intra frame and
        later frames are residuals already subtracted by the caller."""
        xyz = np.ascontiguousarray(xyz, np.float32)
        st = C.c_int(0)
        h = self.lib.pvo_encoder_new(_ptr(xyz, _f32p), xyz.shape[0], 1.0, C.byref(st))
        if not h:
            raise RuntimeError(f"encoder status {st.value}")
        try:
            nl = self.lib.pvo_encoder_leaf_count(h)
            geo = np.zeros(25 + 32 * xyz.shape[0] + 64, np.uint8)
            gsz = self.lib.pvo_encoder_geometry(h, _ptr(geo, _u8p), geo.size)
            cols, coefs = [], []
            for yuv, qp in zip(yuv_frames, qps):
                yuv = np.ascontiguousarray(yuv, np.float32)
                coef = np.zeros((nl, 3), np.float32)
                s = self.lib.pvo_encoder_raht(h, _ptr(yuv, _f32p), _ptr(coef, _f32p))
                if s:
                    raise RuntimeError(f"raht status {s}")
                cap = 64 * nl + 256
                out = np.zeros(cap, np.uint8)
                n = self.lib.pvo_encode_colors(_ptr(coef, _f32p), nl, qp, _ptr(out, _u8p), cap)
                cols.append(out[:n].tobytes())
                coefs.append(coef)
            return geo[:gsz].tobytes(), nl, cols, coefs
        finally:
            self.lib.pvo_encoder_free(h)

    def raht_fp64_error(self, frames: list, parse) -> dict:
        """The FP32 inverse RAHT (the reference's arithmetic, which the GPU
        decoder reproduces bit for bit) against its FP64 restatement on the
        same bitstreams: frames in order, one decoder per patch index.
        Returns the max and mean absolute YUV error, and how many RGB bytes
        (rounded as the CPU decoder rounds them, clamped) the FP32 result
        changes against RGB from the FP64 colours."""
        decs = {}
        mx = 0.0
        tot = 0.0
        cnt = 0
        rgb_diff = 0
        rgb_max = 0
        for b in frames:
            fr = parse(b)
            for i in range(fr.n):
                idx = int(fr.index[i])
                if idx not in decs:
                    decs[idx] = self.decoder()
                    decs[idx].enable_fp64()
                d = decs[idx]
                st = d.set_slice(int(fr.type[i]), int(fr.size[i]), int(fr.qp[i]), fr.geometry[i], fr.color[i])
                if st:
                    raise ValueError(f"slice status {st}")
                _, y32, rgb32 = d.get_patch()
                y64 = d.get_yuv_fp64()
                e = np.abs(y32.astype(np.float64) - y64)
                mx = max(mx, float(e.max()) if e.size else 0.0)
                tot += float(e.sum())
                cnt += e.size
                r64 = _rgb_from_yuv64(y64)
                dd = np.abs(r64.astype(np.int32) - rgb32.astype(np.int32))
                rgb_diff += int((dd != 0).sum())
                rgb_max = max(rgb_max, int(dd.max()) if dd.size else 0)
        return {"yuv_max_abs": mx, "yuv_mean_abs": tot / max(cnt, 1), "values": cnt,
                "rgb_bytes_differing": rgb_diff, "rgb_frac_differing": rgb_diff / max(cnt, 1), "rgb_max_abs": rgb_max}

    # ---- decoder ----
    def decoder(self):
        return OracleDecoder(self)

    def transform(self, mv_rowmajor: np.ndarray, xyz: np.ndarray) -> np.ndarray:
        mv = np.ascontiguousarray(mv_rowmajor, np.float32).reshape(16)
        xyz = np.ascontiguousarray(xyz, np.float32)
        out = np.empty_like(xyz)
        self.lib.pvo_transform(_ptr(mv, _f32p), _ptr(xyz, _f32p), xyz.shape[0], _ptr(out, _f32p))
        return out

    def decode_frame(self, decoders: list, frame, nthreads: int = 1):
        """Decode one parsed frame (pvvc.bitstream.Frame-like: SoA fields with raw
        payloads) through the thread-pool driver.  Returns (xyz, rgb, status)."""
        n = frame.n
        index = np.ascontiguousarray(frame.index, np.int32)
        typ = np.ascontiguousarray(frame.type, np.uint8)
        size = np.ascontiguousarray(frame.size, np.uint32)
        qp = np.ascontiguousarray(frame.qp, np.uint8)
        mv = np.ascontiguousarray(frame.mv, np.float32).reshape(n, 16)
        gsz = np.array([len(g) for g in frame.geometry], np.uint32)
        csz = np.array([len(c) for c in frame.color], np.uint32)
        keep = []
        geo_p = (_u8p * n)()
        col_p = (_u8p * n)()
        for i in range(n):
            g = np.frombuffer(frame.geometry[i] or b"\0", np.uint8).copy()
            c = np.frombuffer(frame.color[i] or b"\0", np.uint8).copy()
            keep += [g, c]
            geo_p[i] = _ptr(g, _u8p) if len(frame.geometry[i]) else None
            col_p[i] = _ptr(c, _u8p) if len(frame.color[i]) else None
        off = np.zeros(n, np.uint64)
        if n:
            off[1:] = np.cumsum(size.astype(np.uint64))[:-1]
        total = int(size.sum())
        xyz = np.zeros((max(total, 1), 3), np.float32)
        rgb = np.zeros((max(total, 1), 3), np.uint8)
        st = np.zeros(max(n, 1), np.int32)
        f = _PvoFrame(n, _ptr(index, _i32p), _ptr(typ, _u8p), _ptr(size, _u32p), _ptr(qp, _u8p), _ptr(mv, _f32p),
                      C.cast(geo_p, C.POINTER(_u8p)), _ptr(gsz, _u32p), C.cast(col_p, C.POINTER(_u8p)), _ptr(csz, _u32p), _ptr(off, _u64p))
        handles = (C.c_void_p * len(decoders))(*[d.h for d in decoders])
        self.lib.pvo_decode_frame(handles, len(decoders), C.byref(f), _ptr(xyz, _f32p), _ptr(rgb, _u8p), _ptr(st, _i32p), nthreads)
        return xyz[:total], rgb[:total], st[:n]

    # ---- ICP ----
    def icp_align(self, src, tgt, init=None, max_corr_dist=1e6, max_iter=50, fitness_eps=1e-6, transform_eps=1e-6, mse_abs_eps=1e-12):
        src = np.ascontiguousarray(src, np.float32)
        tgt = np.ascontiguousarray(tgt, np.float32)
        T = np.zeros(16, np.float32)
        fit = C.c_float(0)
        it = C.c_int(0)
        conv = C.c_int(0)
        p = _IcpParams(max_corr_dist, max_iter, fitness_eps, transform_eps, mse_abs_eps)
        ini = None if init is None else _ptr(np.ascontiguousarray(init, np.float32).reshape(16), _f32p)
        st = self.lib.pvo_icp_align(_ptr(src, _f32p), src.shape[0], _ptr(tgt, _f32p), tgt.shape[0], ini, C.byref(p), _ptr(T, _f32p), C.byref(fit), C.byref(it), C.byref(conv))
        if st:
            raise RuntimeError(f"icp status {st}")
        return T.reshape(4, 4), float(fit.value), int(it.value), bool(conv.value)

    def icp_batch(self, src_list, tgt_list, nthreads, max_corr_dist=1e6, max_iter=50, fitness_eps=0.0,
                  transform_eps=0.0, mse_abs_eps=1e-6):
        """pvo_icp_align over many pairs on nthreads threads."""
        n = len(src_list)
        s = np.ascontiguousarray(np.concatenate(src_list), np.float32)
        t = np.ascontiguousarray(np.concatenate(tgt_list), np.float32)
        so = np.zeros(n + 1, np.uint32); so[1:] = np.cumsum([x.shape[0] for x in src_list])
        to = np.zeros(n + 1, np.uint32); to[1:] = np.cumsum([x.shape[0] for x in tgt_list])
        T = np.zeros((n, 16), np.float32)
        fit = np.zeros(n, np.float32)
        it = np.zeros(n, np.int32)
        cv = np.zeros(n, np.int32)
        p = _IcpParams(max_corr_dist, max_iter, fitness_eps, transform_eps, mse_abs_eps)
        self.lib.pvo_icp_batch(n, _ptr(s, _f32p), _ptr(so, _u32p), _ptr(t, _f32p), _ptr(to, _u32p), C.byref(p),
                               _ptr(T, _f32p), _ptr(fit, _f32p), it.ctypes.data_as(C.POINTER(C.c_int)),
                               cv.ctypes.data_as(C.POINTER(C.c_int)), nthreads)
        return T.reshape(n, 4, 4), fit, it, cv.astype(bool)

    def cloud_mse(self, a, b) -> float:
        a = np.ascontiguousarray(a, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        return float(self.lib.pvo_cloud_mse(_ptr(a, _f32p), a.shape[0], _ptr(b, _f32p), b.shape[0]))

    def fitting_cloud(self, patches, seed: int = 1, clustering_ths: float = 1.0, clustering_err_ths: float = 0.1,
                      max_iter: int = 100):
        """PatchFitting::Compute (direct clustering) of the GoP's registered
        patches: (the fitting cloud float32 [m,3], {cells, iterations})."""
        arrs = [np.ascontiguousarray(x, np.float32).reshape(-1, 3) for x in patches]
        ptrs = (_f32p * len(arrs))(*[_ptr(a, _f32p) for a in arrs])
        ns = np.array([a.shape[0] for a in arrs], np.uint32)
        cap = int(ns.sum()) + 16
        out = np.zeros((cap, 3), np.float32)
        st = (C.c_long * 3)()
        k = self.lib.pvo_fitting_cloud(len(arrs), ptrs, _ptr(ns, _u32p), clustering_ths, clustering_err_ths, max_iter, seed,
                                       _ptr(out, _f32p), cap, st)
        if k < 0:
            raise RuntimeError(f"fitting_cloud status {-k}")
        return out[:k], {"cells": int(st[0]), "iterations": int(st[1]), "empty_redraws": int(st[2])}

    def cloud_quality(self, p_xyz, p_rgb, q_xyz, q_rgb, brute: bool = False) -> np.ndarray:
        """common::MSE::Compute of p against q: [geo p->q, geo q->p, Y, Y, U, U, V, V]."""
        a = np.ascontiguousarray(p_xyz, np.float32).reshape(-1, 3)
        ac = np.ascontiguousarray(p_rgb, np.uint8).reshape(-1, 3)
        b = np.ascontiguousarray(q_xyz, np.float32).reshape(-1, 3)
        bc = np.ascontiguousarray(q_rgb, np.uint8).reshape(-1, 3)
        out = np.zeros(8, np.float64)
        st = self.lib.pvo_cloud_quality(_ptr(a, _f32p), _ptr(ac, _u8p), a.shape[0], _ptr(b, _f32p), _ptr(bc, _u8p),
                                        b.shape[0], 1 if brute else 0, out.ctypes.data_as(C.POINTER(C.c_double)))
        if st:
            raise RuntimeError(f"cloud_quality status {st}")
        return out

    # ---- colour interpolation (GoP_encoding.cc:73-95,131-150) ----
    def knn_colors(self, q, src, rgb, k=10, brute=False) -> np.ndarray:
        """YUV [nq,3] interpolated at the query points from the k nearest
        source points (pvo_knn_colors)."""
        q = np.ascontiguousarray(q, np.float32).reshape(-1, 3)
        src = np.ascontiguousarray(src, np.float32).reshape(-1, 3)
        rgb = np.ascontiguousarray(rgb, np.uint8).reshape(-1, 3)
        out = np.zeros((max(q.shape[0], 1), 3), np.float32)
        st = self.lib.pvo_knn_colors(_ptr(q, _f32p), q.shape[0], _ptr(src, _f32p), _ptr(rgb, _u8p), src.shape[0], k,
                                     1 if brute else 0, _ptr(out, _f32p))
        if st:
            raise RuntimeError(f"knn status {st}")
        return out[:q.shape[0]]

    def knn_colors_batch(self, queries, sources, rgbs, k, nthreads) -> list:
        """knn_colors over many (query, source) pairs on nthreads threads."""
        n = len(sources)
        q = np.ascontiguousarray(np.concatenate(queries), np.float32)
        qn = np.array([x.shape[0] for x in queries], np.uint32)
        qoff = np.zeros(n, np.uint64); qoff[1:] = np.cumsum(qn.astype(np.uint64))[:-1]
        s = np.ascontiguousarray(np.concatenate(sources), np.float32)
        c = np.ascontiguousarray(np.concatenate(rgbs), np.uint8)
        so = np.zeros(n + 1, np.uint32); so[1:] = np.cumsum([x.shape[0] for x in sources])
        out = np.zeros((max(int(qn.sum()), 1), 3), np.float32)
        st = self.lib.pvo_knn_colors_batch(n, _ptr(q, _f32p), qoff.ctypes.data_as(C.POINTER(C.c_uint64)), _ptr(qn, _u32p),
                                           _ptr(s, _f32p), _ptr(c, _u8p), _ptr(so, _u32p), k, _ptr(out, _f32p),
                                           qoff.ctypes.data_as(C.POINTER(C.c_uint64)), nthreads)
        if st:
            raise RuntimeError(f"knn status {st}")
        return [out[int(a):int(a) + int(m)] for a, m in zip(qoff, qn)]


def _rgb_from_yuv64(yuv: np.ndarray) -> np.ndarray:
    """BT.601 YUV->RGB of common.h:154-158 evaluated in double, rounded half
    away from zero and clamped to [0, 255]."""
    y, u, v = yuv[:, 0], yuv[:, 1], yuv[:, 2]
    rgb = np.stack([y + 1.402 * (v - 128), y - 0.3441 * (u - 128) - 0.7141 * (v - 128), y + 1.772 * (u - 128)], 1)
    r = np.sign(rgb) * np.floor(np.abs(rgb) + 0.5)
    return np.clip(r, 0, 255).astype(np.uint8)


class OracleDecoder:
    """One persistent per-patch-index decoder (InvertRAHTOctree)."""

    def __init__(self, o: Oracle):
        self.o = o
        self.h = o.lib.pvo_decoder_new()

    def __del__(self):
        try:
            self.o.lib.pvo_decoder_free(self.h)
        except Exception:
            pass

    def set_slice(self, type_, size, qp, geo: bytes, col: bytes) -> int:
        g = np.frombuffer(geo or b"\0", np.uint8).copy()
        c = np.frombuffer(col or b"\0", np.uint8).copy()
        return self.o.lib.pvo_decoder_set_slice(self.h, type_, size, qp, _ptr(g, _u8p) if geo else None, len(geo or b""),
                                                _ptr(c, _u8p) if col else None, len(col or b""))

    def get_patch(self):
        n = self.o.lib.pvo_decoder_size(self.h)
        xyz = np.zeros((max(n, 1), 3), np.float32)
        yuv = np.zeros((max(n, 1), 3), np.float32)
        rgb = np.zeros((max(n, 1), 3), np.uint8)
        s = self.o.lib.pvo_decoder_get_patch(self.h, _ptr(xyz, _f32p), _ptr(yuv, _f32p), _ptr(rgb, _u8p))
        if s:
            raise ValueError(f"get_patch status {s}")
        return xyz[:n], yuv[:n], rgb[:n]

    def enable_fp64(self, on: bool = True):
        """Also run the FP64 restatement of the inverse RAHT on every slice
        (enable before the slot's intra slice)."""
        self.o.lib.pvo_decoder_enable_fp64(self.h, 1 if on else 0)

    def get_yuv_fp64(self) -> np.ndarray:
        n = self.o.lib.pvo_decoder_size(self.h)
        yuv = np.zeros((max(n, 1), 3), np.float64)
        s = self.o.lib.pvo_decoder_get_yuv_fp64(self.h, yuv.ctypes.data_as(C.POINTER(C.c_double)))
        if s:
            raise ValueError(f"get_yuv_fp64 status {s}")
        return yuv[:n]


class Reference:
    """The reference's own codec classes (compiled against shims).  Only
    available where the reference tree is present (this build container)."""

    def __init__(self):
        so = build_reference()
        if so is None:
            raise RuntimeError("reference sources not available on this machine")
        lib = C.CDLL(so)
        self.lib = lib
        lib.ref_rlgr_encode.restype = C.c_long
        lib.ref_rlgr_encode.argtypes = [_i64p, C.c_size_t, _u8p, C.c_size_t]
        lib.ref_rlgr_decode.restype = C.c_long
        lib.ref_rlgr_decode.argtypes = [_u8p, C.c_size_t, C.c_size_t, _i64p]
        lib.ref_zstd_encode.restype = C.c_long
        lib.ref_zstd_encode.argtypes = [_u8p, C.c_size_t, C.c_int, _u8p, C.c_size_t]
        lib.ref_zstd_decode.restype = C.c_long
        lib.ref_zstd_decode.argtypes = [_u8p, C.c_size_t, _u8p, C.c_size_t]
        lib.ref_encoder_new.restype = C.c_void_p
        lib.ref_encoder_new.argtypes = [_f32p, C.c_size_t]
        lib.ref_encoder_free.argtypes = [C.c_void_p]
        lib.ref_encoder_geometry.restype = C.c_long
        lib.ref_encoder_geometry.argtypes = [C.c_void_p, _u8p, C.c_size_t]
        lib.ref_encoder_raht.restype = C.c_long
        lib.ref_encoder_raht.argtypes = [C.c_void_p, _f32p, C.c_size_t, _f32p, C.c_size_t]
        lib.ref_decoder_new.restype = C.c_void_p
        lib.ref_decoder_free.argtypes = [C.c_void_p]
        lib.ref_decoder_set_slice.restype = C.c_int
        lib.ref_decoder_set_slice.argtypes = [C.c_void_p, C.c_uint8, C.c_int, C.c_int, C.c_uint64, C.c_uint8, _f32p, _u8p, C.c_size_t, _u8p, C.c_size_t]
        lib.ref_decoder_get_patch.restype = C.c_long
        lib.ref_decoder_get_patch.argtypes = [C.c_void_p, _f32p, _u8p, C.c_size_t]
        lib.ref_cloud_mse.restype = C.c_float
        lib.ref_cloud_mse.argtypes = [_f32p, C.c_size_t, _f32p, C.c_size_t]
        lib.ref_fitting_cloud.restype = C.c_long
        lib.ref_fitting_cloud.argtypes = [C.c_int, C.POINTER(_f32p), _u32p, C.c_float, C.c_float, C.c_int, C.c_uint, _f32p,
                                          C.c_size_t]
        lib.ref_mse_compute.restype = C.c_int
        lib.ref_mse_compute.argtypes = [_f32p, _u8p, C.c_size_t, _f32p, _u8p, C.c_size_t, C.POINTER(C.c_double)]
        lib.ref_gop_encode.restype = C.c_int
        lib.ref_gop_encode.argtypes = [_f32p, C.c_size_t, C.c_int, C.POINTER(_f32p), C.POINTER(_u8p),
                                       C.POINTER(C.c_size_t), C.c_int, C.c_int, C.c_int, _f32p, _u8p, C.c_size_t,
                                       C.POINTER(C.c_size_t), _u8p, C.c_size_t, C.POINTER(C.c_size_t)]
        lib.ref_save_slice.restype = C.c_int
        lib.ref_save_slice.argtypes = [C.c_char_p, C.c_uint8, C.c_int, C.c_int, C.c_uint64, C.c_uint8, _f32p, _u8p, C.c_size_t, _u8p, C.c_size_t]
        lib.ref_change_slice_to_frame.restype = C.c_int
        lib.ref_change_slice_to_frame.argtypes = [C.c_char_p, C.c_char_p]


    def cloud_mse(self, a, b) -> float:
        """ICPBase::CloudMSE of cloud a (transformed source) against b."""
        a = np.ascontiguousarray(a, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        return float(self.lib.ref_cloud_mse(_ptr(a, _f32p), a.shape[0], _ptr(b, _f32p), b.shape[0]))

    def fitting_cloud(self, patches, seed: int = 1, clustering_ths: float = 1.0, clustering_err_ths: float = 0.1,
                      max_iter: int = 100) -> np.ndarray:
        """The reference's PatchFitting::Compute after srand(seed)."""
        arrs = [np.ascontiguousarray(x, np.float32).reshape(-1, 3) for x in patches]
        ptrs = (_f32p * len(arrs))(*[_ptr(a, _f32p) for a in arrs])
        ns = np.array([a.shape[0] for a in arrs], np.uint32)
        cap = int(ns.sum()) + 16
        out = np.zeros((cap, 3), np.float32)
        k = self.lib.ref_fitting_cloud(len(arrs), ptrs, _ptr(ns, _u32p), clustering_ths, clustering_err_ths, max_iter, seed,
                                       _ptr(out, _f32p), cap)
        if k < 0:
            raise RuntimeError(f"reference PatchFitting status {k}")
        return out[:k]

    def mse_compute(self, p_xyz, p_rgb, q_xyz, q_rgb) -> np.ndarray:
        """The reference's common::MSE::Compute: [geo p->q, geo q->p, Y, Y, U, U, V, V]."""
        a = np.ascontiguousarray(p_xyz, np.float32).reshape(-1, 3)
        ac = np.ascontiguousarray(p_rgb, np.uint8).reshape(-1, 3)
        b = np.ascontiguousarray(q_xyz, np.float32).reshape(-1, 3)
        bc = np.ascontiguousarray(q_rgb, np.uint8).reshape(-1, 3)
        out = np.zeros(8, np.float64)
        if self.lib.ref_mse_compute(_ptr(a, _f32p), _ptr(ac, _u8p), a.shape[0], _ptr(b, _f32p), _ptr(bc, _u8p), b.shape[0],
                                    out.ctypes.data_as(C.POINTER(C.c_double))):
            raise RuntimeError("reference MSE::Compute threw")
        return out

    def gop_encode(self, fit_xyz, srcs, rgbs, k, qp_i, qp_p):
        """GoPEncoding::Encode on one patch's GoP (ref_gop_encode): the
        interpolated colours [nf,n,3] (later frames as residuals), the
        geometry payload and the raw colour payload of every frame."""
        fit = np.ascontiguousarray(fit_xyz, np.float32)
        n, nf = fit.shape[0], len(srcs)
        srcs = [np.ascontiguousarray(x, np.float32) for x in srcs]
        rgbs = [np.ascontiguousarray(x, np.uint8) for x in rgbs]
        sp = (_f32p * nf)(*[_ptr(x, _f32p) for x in srcs])
        cp = (_u8p * nf)(*[_ptr(x, _u8p) for x in rgbs])
        sn = (C.c_size_t * nf)(*[x.shape[0] for x in srcs])
        cols = np.zeros((nf, n, 3), np.float32)
        geo = np.zeros(64 + 4 * n, np.uint8)
        pay = np.zeros(nf * (64 + 16 * n), np.uint8)
        gl = C.c_size_t(0)
        cl = (C.c_size_t * nf)()
        rc = self.lib.ref_gop_encode(_ptr(fit, _f32p), n, nf, sp, cp, sn, k, qp_i, qp_p, _ptr(cols, _f32p),
                                     _ptr(geo, _u8p), geo.size, C.byref(gl), _ptr(pay, _u8p), pay.size, cl)
        if rc:
            raise RuntimeError(f"ref_gop_encode {rc}")
        off = np.concatenate([[0], np.cumsum(list(cl))]).astype(np.int64)
        return cols, geo[:gl.value].tobytes(), [pay[off[f]:off[f + 1]].tobytes() for f in range(nf)]
    def rlgr_encode(self, sym) -> bytes:
        sym = np.ascontiguousarray(sym, np.int64)
        cap = 16 * sym.size + 64
        out = np.zeros(cap, np.uint8)
        n = self.lib.ref_rlgr_encode(_ptr(sym, _i64p), sym.size, _ptr(out, _u8p), cap)
        if n < 0:
            raise RuntimeError("reference rlgr encode failed")
        return out[:n].tobytes()

    def rlgr_decode(self, data: bytes, nsym: int) -> np.ndarray:
        buf = np.frombuffer(data, np.uint8).copy()
        out = np.zeros(max(nsym, 1), np.int64)
        n = self.lib.ref_rlgr_decode(_ptr(buf, _u8p), len(data), nsym, _ptr(out, _i64p))
        if n < 0:
            raise RuntimeError("reference rlgr decode failed")
        return out[:nsym]

    def zstd_encode(self, data: bytes, level: int = 22) -> bytes:
        src = np.frombuffer(data, np.uint8).copy()
        cap = len(data) * 2 + 1024
        out = np.zeros(cap, np.uint8)
        n = self.lib.ref_zstd_encode(_ptr(src, _u8p), len(data), level, _ptr(out, _u8p), cap)
        if n < 0:
            raise RuntimeError("zstd encode failed")
        return out[:n].tobytes()

    def encode_patch(self, xyz, yuv_frames, qps, oracle_quantise):
        """Geometry + per-frame RAHT coefficients from the reference classes;
        the quantise+RLGR step uses the reference RLGR encoder on the
        GoP_encoding.cc:184-189 quantisation done here in float32."""
        xyz = np.ascontiguousarray(xyz, np.float32)
        h = self.lib.ref_encoder_new(_ptr(xyz, _f32p), xyz.shape[0])
        if not h:
            raise RuntimeError("reference encoder failed")
        try:
            geo = np.zeros(25 + 32 * xyz.shape[0] + 64, np.uint8)
            gsz = self.lib.ref_encoder_geometry(h, _ptr(geo, _u8p), geo.size)
            cols, coefs = [], []
            for yuv, qp in zip(yuv_frames, qps):
                yuv = np.ascontiguousarray(yuv, np.float32)
                coef = np.zeros((xyz.shape[0], 3), np.float32)
                nl = self.lib.ref_encoder_raht(h, _ptr(yuv, _f32p), xyz.shape[0], _ptr(coef, _f32p), xyz.shape[0])
                coef = coef[:nl]
                sym = oracle_quantise(coef, qp)
                cols.append(self.rlgr_encode(sym))
                coefs.append(coef)
            return geo[:gsz].tobytes(), nl, cols, coefs
        finally:
            self.lib.ref_encoder_free(h)

    def decoder(self):
        return RefDecoder(self)


def quantise(coef: np.ndarray, qp: int) -> np.ndarray:
    """GoP_encoding.cc:184-189 in float32: round(c / QP) as int64, planes Y||U||V."""
    c = np.ascontiguousarray(coef, np.float32)
    q = np.round(c / np.float32(qp)).astype(np.int64)  # numpy rounds half to even
    # std::round rounds half away from zero: fix the exact .5 cases
    d = (c / np.float32(qp)).astype(np.float32)
    half = np.abs(d - np.trunc(d)) == 0.5
    q[half] = (np.trunc(d[half]) + np.sign(d[half])).astype(np.int64)
    return np.concatenate([q[:, 0], q[:, 1], q[:, 2]])


class RefDecoder:
    def __init__(self, r: Reference):
        self.r = r
        self.h = r.lib.ref_decoder_new()

    def __del__(self):
        try:
            self.r.lib.ref_decoder_free(self.h)
        except Exception:
            pass

    def set_slice(self, type_, size, qp, geo: bytes, col: bytes, mv_colmajor=None, timestamp=0, index=0) -> int:
        mv = np.eye(4, dtype=np.float32).reshape(16) if mv_colmajor is None else np.ascontiguousarray(mv_colmajor, np.float32).reshape(16)
        g = np.frombuffer(geo or b"\0", np.uint8).copy()
        c = np.frombuffer(col or b"\0", np.uint8).copy()
        return self.r.lib.ref_decoder_set_slice(self.h, type_, timestamp, index, size, qp, _ptr(mv, _f32p),
                                                _ptr(g, _u8p) if geo else None, len(geo or b""), _ptr(c, _u8p) if col else None, len(col or b""))

    def get_patch(self, cap: int):
        xyz = np.zeros((cap, 3), np.float32)
        rgb = np.zeros((cap, 3), np.uint8)
        n = self.r.lib.ref_decoder_get_patch(self.h, _ptr(xyz, _f32p), _ptr(rgb, _u8p), cap)
        if n < 0:
            raise RuntimeError("reference get_patch failed")
        return xyz[:n], rgb[:n]
