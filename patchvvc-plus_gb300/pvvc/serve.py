"""Playback serving over the C ABI's pvvc_server_*: many concurrent streams
of .frame requests decoded with continuous batching on one GPU.  It stands
where the reference client's decode thread stands
(src/cuda/common/manager.cc:230-270, one stream, one frame per launch).

  Server     the C-ABI server (admission by HBM budget, submit/poll/release)
  playback   a load generator: per-stream Poisson frame arrivals at a jittered
             frame rate, submitted in real time; returns per-frame latencies
"""
from __future__ import annotations

import ctypes as C
import threading
import time

import numpy as np

from . import _lib as L
from .codec import _tune


class Server:
    def __init__(self, hbm_budget_bytes: int, max_leaves: int = 8192, max_nodes: int | None = None,
                 max_batch_points: int = 32 << 20, ring_points: int = 256 << 20, inflight: int = 2,
                 max_batch_frames: int = 4096, tune=None):
        cfg = L.ServerConfig(int(hbm_budget_bytes), int(max_leaves), int(max_nodes or 2 * max_leaves),
                             int(max_batch_points), int(ring_points), int(inflight), int(max_batch_frames), _tune(tune))
        h = L.vp()
        L.check(L.lib().pvvc_server_create(C.byref(cfg), C.byref(h)), "pvvc_server_create")
        self.h = h
        self._lock = threading.Lock()
        self._live = {}      # internal tag -> (user tag, bytes kept alive until completion)
        self._seq = 0
        self._buf = (L.Completion * 4096)()

    def open_stream(self, nslots: int) -> int:
        sid = C.c_int32(-1)
        L.check(L.lib().pvvc_server_open_stream(self.h, int(nslots), C.byref(sid)), "pvvc_server_open_stream")
        return int(sid.value)

    def try_open_stream(self, nslots: int):
        """Stream id, or None when the HBM budget cannot hold the stream now."""
        sid = C.c_int32(-1)
        rc = L.lib().pvvc_server_open_stream(self.h, int(nslots), C.byref(sid))
        if rc == 11:
            return None
        L.check(rc, "pvvc_server_open_stream")
        return int(sid.value)

    def close_stream(self, sid: int) -> None:
        L.check(L.lib().pvvc_server_close_stream(self.h, int(sid)), "pvvc_server_close_stream")

    def submit(self, sid: int, frame: bytes, tag=None) -> None:
        buf = np.frombuffer(frame, np.uint8)
        with self._lock:
            self._seq += 1
            k = self._seq
            self._live[k] = (tag, buf)
        rc = L.lib().pvvc_server_submit(self.h, int(sid), buf.ctypes.data, buf.size, k)
        if rc:
            with self._lock:
                self._live.pop(k, None)
            raise L.PvvcError(rc, "pvvc_server_submit")

    def poll(self, wait_us: int = 1000) -> list[dict]:
        n = C.c_int32(0)
        L.check(L.lib().pvvc_server_poll(self.h, self._buf, len(self._buf), C.byref(n), int(wait_us)), "pvvc_server_poll")
        out = []
        with self._lock:
            for i in range(n.value):
                c = self._buf[i]
                tag, _ = self._live.pop(int(c.tag), (None, None))
                out.append({"tag": tag, "handle": int(c.handle), "stream": int(c.stream_id), "status": int(c.status),
                            "npoints": int(c.npoints), "xyz": c.xyz, "rgb": c.rgb, "submit_us": c.submit_us,
                            "launch_us": c.launch_us, "done_us": c.done_us, "batch": int(c.batch_id),
                            "batch_frames": int(c.batch_frames)})
        return out

    def read(self, comp: dict):
        n = comp["npoints"]
        xyz = np.zeros((max(n, 1), 3), np.float32)
        rgb = np.zeros((max(n, 1), 3), np.uint8)
        L.check(L.lib().pvvc_server_read(self.h, comp["handle"], xyz.ctypes.data_as(L.f32p), rgb.ctypes.data_as(L.u8p)),
                "pvvc_server_read")
        return xyz[:n], rgb[:n]

    def release(self, comp: dict) -> None:
        L.check(L.lib().pvvc_server_release(self.h, comp["handle"]), "pvvc_server_release")

    def stats(self) -> dict:
        s = L.ServerStats()
        L.check(L.lib().pvvc_server_stats_get(self.h, C.byref(s)), "pvvc_server_stats_get")
        return {k: (float(getattr(s, k)) if k == "gpu_busy_us" else int(getattr(s, k))) for k, _ in L.ServerStats._fields_}

    def close(self):
        if self.h:
            L.lib().pvvc_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def slots_needed(frames: list[bytes]) -> int:
    from .frame import parse_frame
    m = 0
    for b in frames:
        f = parse_frame(b)
        if f.n:
            m = max(m, int(f.index.max()) + 1)
    return max(m, 1)


def arrival_schedule(nstreams: int, duration_s: float, fps: float = 30.0, jitter: float = 0.2, seed: int = 0):
    """(time_s, stream, k) of every request: stream i requests its frames k =
    0, 1, ... as a Poisson process of rate fps * U(1-jitter, 1+jitter)."""
    rng = np.random.default_rng(seed)
    ev = []
    for i in range(nstreams):
        rate = fps * rng.uniform(1 - jitter, 1 + jitter)
        t, k = rng.exponential(1 / rate), 0
        while t < duration_s:
            ev.append((t, i, k))
            k += 1
            t += rng.exponential(1 / rate)
    ev.sort()
    return ev


def playback(server: Server, streams: list[list[bytes]], duration_s: float, fps: float = 30.0, jitter: float = 0.2,
             seed: int = 0, warmup_s: float = 1.0, keep=None) -> dict:
    """Real-time playback of `streams` (each a list of .frame bytes starting at
    an intra frame, looped) against `server`.  Every stream is opened first
    (admission); requests are submitted at their arrival times by a submitter
    thread while this thread polls, releases and records completions.
    keep(stream, k, completion) may read a completion before its release."""
    sids = [server.open_stream(slots_needed(fr)) for fr in streams]
    ev = arrival_schedule(len(streams), duration_s, fps, jitter, seed)
    total = len(ev)
    err = []

    def submitter():
        t0 = time.perf_counter()
        try:
            for t, i, k in ev:
                dt = t - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                fr = streams[i]
                server.submit(sids[i], fr[k % len(fr)], tag=(i, k, t))
        except Exception as e:  # surfaced by the caller
            err.append(e)

    th = threading.Thread(target=submitter, daemon=True)
    wall0 = time.perf_counter()
    th.start()
    got = []
    deadline = time.perf_counter() + duration_s + 60
    while len(got) < total and time.perf_counter() < deadline:
        if err:
            break
        for c in server.poll(wait_us=2000):
            i, k, t = c["tag"]
            if keep is not None:
                keep(i, k, c)
            server.release(c)
            got.append((i, k, t, c["status"], c["npoints"], c["submit_us"], c["launch_us"], c["done_us"],
                        c["batch"], c["batch_frames"]))
    th.join(timeout=5)
    wall = time.perf_counter() - wall0
    for sid in sids:
        server.close_stream(sid)
    if err:
        raise err[0]
    a = np.array([g[3:] for g in got], np.float64).reshape(-1, 7)
    t_arr = np.array([g[2] for g in got])
    lat_ms = (a[:, 4] - a[:, 2]) / 1e3
    steady = t_arr >= warmup_s
    lat = lat_ms[steady] if steady.any() else lat_ms
    span_us = a[:, 4].max() - a[:, 2].min() if len(a) else 1.0
    st = server.stats()
    bad = [(g[0], g[1], g[3], g[9]) for g in got if g[3] != 0]
    hist = {}
    for _, _, code, _ in bad:
        hist[int(code)] = hist.get(int(code), 0) + 1
    diag = {"error_status": hist,
            "error_samples": [{"stream": int(i), "frame": int(k % len(streams[i])), "k": int(k), "status": int(code),
                               "batch_frames": int(bf)} for i, k, code, bf in bad[:12]]}
    return {**diag, "streams": len(streams), "requests": total, "completed": len(got), "errors": int((a[:, 0] != 0).sum()),
            "p50_ms": float(np.percentile(lat, 50)), "p95_ms": float(np.percentile(lat, 95)),
            "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max()), "mean_ms": float(lat.mean()),
            "points": int(a[:, 1].sum()), "mpts_per_s": float(a[:, 1].sum() / (span_us / 1e6) / 1e6),
            "wall_s": wall, "batches": int(len(np.unique(a[:, 5]))), "mean_batch_frames": float(a[:, 6].mean()),
            "gpu_busy_frac": float(st["gpu_busy_us"] / span_us) if span_us > 0 else 0.0,
            "reserved_gb": st["reserved_bytes"] / 1e9, "slots_total": st["slots_total"]}
