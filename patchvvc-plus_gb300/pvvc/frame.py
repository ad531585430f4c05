"""Host-side view of .frame / .slice bytes (layouts of src/io/slice_io.cc:20-322
and src/cuda/common/slice_io.cu:143-275) and packing of frames into one
device batch (payload bytes + per-slice descriptors)."""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

TYPE_VALID, TYPE_PREDICT, TYPE_SKIP, TYPE_GEO_ZSTD, TYPE_COLOR_ZSTD = 0x01, 0x02, 0x04, 0x08, 0x10


@dataclass
class Frame:
    timestamp: int
    index: np.ndarray          # int32 [n]
    type: np.ndarray           # uint8 [n]
    size: np.ndarray           # uint32 [n]
    qp: np.ndarray             # uint8 [n]
    mv: np.ndarray             # float32 [n,16] row-major
    geometry: list = field(default_factory=list)  # bytes per slice (b"" for predictive)
    color: list = field(default_factory=list)

    @property
    def n(self) -> int:
        return int(self.index.shape[0])

    @property
    def points(self) -> int:
        return int(self.size.astype(np.int64).sum())


def parse_frame(b: bytes) -> Frame:
    """io::LoadFrame without the zstd step."""
    mv_ = memoryview(b)
    ts, n = struct.unpack_from("<iI", b, 0)
    o = 8
    if n * 82 > len(b):
        raise ValueError("malformed frame: slice count")
    index = np.frombuffer(mv_[o:o + 4 * n], np.int32).copy(); o += 4 * n
    typ = np.frombuffer(mv_[o:o + n], np.uint8).copy(); o += n
    size = np.frombuffer(mv_[o:o + 4 * n], np.uint32).copy(); o += 4 * n
    qp = np.frombuffer(mv_[o:o + n], np.uint8).copy(); o += n
    mv = np.frombuffer(mv_[o:o + 64 * n], np.float32).reshape(n, 16).copy(); o += 64 * n
    gsz = np.frombuffer(mv_[o:o + 4 * n], np.uint32); o += 4 * n
    geo = []
    for i in range(n):
        g = int(gsz[i])
        if o + g > len(b):
            raise ValueError("malformed frame: geometry")
        geo.append(bytes(mv_[o:o + g])); o += g
    csz = np.frombuffer(mv_[o:o + 4 * n], np.uint32); o += 4 * n
    col = []
    for i in range(n):
        c = int(csz[i])
        if o + c > len(b):
            raise ValueError("malformed frame: colour")
        col.append(bytes(mv_[o:o + c])); o += c
    return Frame(ts, index, typ, size, qp, mv, geo, col)


def write_frame(f: Frame) -> bytes:
    n = f.n
    parts = [struct.pack("<iI", f.timestamp, n), f.index.astype(np.int32).tobytes(), f.type.astype(np.uint8).tobytes(),
             f.size.astype(np.uint32).tobytes(), f.qp.astype(np.uint8).tobytes(),
             np.ascontiguousarray(f.mv, np.float32).tobytes(),
             np.array([len(g) for g in f.geometry], np.uint32).tobytes(), b"".join(f.geometry),
             np.array([len(c) for c in f.color], np.uint32).tobytes(), b"".join(f.color)]
    return b"".join(parts)


def parse_slice(b: bytes) -> dict:
    """io::LoadSlice: returns a dict with column-major mv as stored."""
    typ, ts, idx, size, qp = struct.unpack_from("<BiiQB", b, 0)
    o = 18
    mv = np.frombuffer(b[o:o + 64], np.float32).copy(); o += 64
    geo = b""
    if not typ & TYPE_PREDICT:
        (g,) = struct.unpack_from("<Q", b, o); o += 8
        geo = b[o:o + g]; o += g
    col = b""
    if not typ & TYPE_SKIP:
        (c,) = struct.unpack_from("<Q", b, o); o += 8
        col = b[o:o + c]; o += c
    return dict(type=typ, timestamp=ts, index=idx, size=size, qp=qp, mv_colmajor=mv, geometry=geo, color=col)


def _align(x: int, a: int = 4) -> int:
    return (x + a - 1) // a * a


@dataclass
class Batch:
    """Slices of several frames packed for one device decode: the payload
    bytes (4-byte aligned per payload) and the per-slice descriptor arrays
    of pvvc_batch_desc."""
    payload: np.ndarray
    slot: np.ndarray
    type: np.ndarray
    size: np.ndarray
    qp: np.ndarray
    mv: np.ndarray
    geo_off: np.ndarray
    geo_size: np.ndarray
    col_off: np.ndarray
    col_size: np.ndarray
    out_off: np.ndarray
    frame_first_slice: np.ndarray   # [nframes+1]
    frame_first_point: np.ndarray   # [nframes+1]

    @property
    def nslices(self) -> int:
        return int(self.slot.shape[0])

    @property
    def points(self) -> int:
        return int(self.frame_first_point[-1])

    @property
    def algorithmic_bytes(self) -> int:
        """Bytes the decode must move at minimum: payload in, 16 floats of mv
        per slice in, xyz (12 B) + rgb (3 B) per point out."""
        return int(self.geo_size.sum() + self.col_size.sum() + 64 * self.nslices + 15 * self.points)


def pack_frames(frames: list[Frame], slot_base: int = 0) -> Batch:
    """Pack frames (raw payloads: pvvc.zstd.inflate_device inflates zstd ones) into one batch.  The
    slot of a slice is slot_base + its patch index."""
    nsl = sum(f.n for f in frames)
    tot = sum(_align(len(g)) + _align(len(c)) for f in frames for g, c in zip(f.geometry, f.color))
    payload = np.zeros(tot + 16, np.uint8)  # the decoder reads whole 16-byte blocks
    slot = np.empty(nsl, np.int32); typ = np.empty(nsl, np.uint8); size = np.empty(nsl, np.uint32)
    qp = np.empty(nsl, np.uint8); mv = np.empty((nsl, 16), np.float32)
    goff = np.zeros(nsl, np.uint64); gsz = np.zeros(nsl, np.uint32)
    coff = np.zeros(nsl, np.uint64); csz = np.zeros(nsl, np.uint32); oo = np.zeros(nsl, np.uint64)
    ffs = [0]; ffp = [0]
    k = 0; off = 0; po = 0
    for f in frames:
        for i in range(f.n):
            if f.type[i] & (TYPE_GEO_ZSTD | TYPE_COLOR_ZSTD):
                raise ValueError("pack_frames wants raw payloads (inflate zstd payloads first)")
            slot[k] = slot_base + int(f.index[i]); typ[k] = f.type[i]; size[k] = f.size[i]; qp[k] = f.qp[i]
            mv[k] = f.mv[i]
            g = f.geometry[i]; c = f.color[i]
            goff[k] = off; gsz[k] = len(g)
            payload[off:off + len(g)] = np.frombuffer(g, np.uint8); off = _align(off + len(g))
            coff[k] = off; csz[k] = len(c)
            payload[off:off + len(c)] = np.frombuffer(c, np.uint8); off = _align(off + len(c))
            oo[k] = po; po += int(f.size[i])
            k += 1
        ffs.append(k); ffp.append(po)
    return Batch(payload, slot, typ, size, qp, mv, goff, gsz, coff, csz, oo, np.array(ffs, np.int64),
                 np.array(ffp, np.int64))


def concat_batches(batches: list[Batch], slot_stride: int) -> Batch:
    """Several independent batches (e.g. GoPs decoded concurrently) in one:
    batch b uses slots [b*slot_stride, (b+1)*slot_stride)."""
    pay, po, so = [], 0, 0
    fields = {k: [] for k in ("slot", "type", "size", "qp", "mv", "geo_off", "geo_size", "col_off", "col_size", "out_off")}
    ffs, ffp = [0], [0]
    off = 0
    for b_i, b in enumerate(batches):
        pay.append(b.payload)
        fields["slot"].append(b.slot + b_i * slot_stride)
        for k in ("type", "size", "qp", "mv", "geo_size", "col_size"):
            fields[k].append(getattr(b, k))
        fields["geo_off"].append(b.geo_off + np.uint64(off))
        fields["col_off"].append(b.col_off + np.uint64(off))
        fields["out_off"].append(b.out_off + np.uint64(po))
        ffs.extend((b.frame_first_slice[1:] + so).tolist())
        ffp.extend((b.frame_first_point[1:] + po).tolist())
        off += b.payload.shape[0]
        po += b.points
        so += b.nslices
    cat = {k: np.concatenate(v) for k, v in fields.items()}
    return Batch(np.concatenate(pay), cat["slot"].astype(np.int32), cat["type"], cat["size"], cat["qp"], cat["mv"],
                 cat["geo_off"], cat["geo_size"], cat["col_off"], cat["col_size"], cat["out_off"],
                 np.array(ffs, np.int64), np.array(ffp, np.int64))
