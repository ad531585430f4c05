"""zstd payloads: the GPU batch inflater and its host build
(pvvc_zstd_inflate_batch / pvvc_zstd_inflate_host), which replace the
reference loader's host ZSTD_decompress (ZstdDecoder::Decode,
src/common/entropy_codec.cc:341-360)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

UNKNOWN = (1 << 64) - 1


def content_size(data: bytes) -> int:
    """ZSTD_getFrameContentSize of the first frame (0 for a skippable frame,
    UNKNOWN when undeclared).  Raises PvvcError on a malformed header."""
    buf = np.frombuffer(data, np.uint8) if len(data) else np.zeros(1, np.uint8)
    out = C.c_uint64(0)
    L.check(L.lib().pvvc_zstd_content_size(buf.ctypes.data_as(L.u8p), len(data), C.byref(out)), "zstd_content_size")
    return out.value


def inflate_host(data: bytes, cap: int) -> bytes:
    """The decoder on the host, ZSTD_decompress(dst, cap, data) semantics."""
    src = np.frombuffer(data, np.uint8) if len(data) else np.zeros(1, np.uint8)
    dst = np.zeros(max(cap, 1), np.uint8)
    n = C.c_uint64(0)
    L.check(L.lib().pvvc_zstd_inflate_host(src.ctypes.data_as(L.u8p), len(data), dst.ctypes.data_as(L.u8p), cap,
                                           C.byref(n)), "zstd_inflate_host")
    return dst[:n.value].tobytes()


def inflate_device(payloads: list[bytes], caps: list[int], stream=None):
    """Inflate every payload on the GPU in one launch.  Returns (outputs,
    statuses): outputs[j] is the inflated bytes (b"" on failure), statuses[j]
    the PVVC status."""
    import torch
    n = len(payloads)
    src_len = np.array([len(p) for p in payloads], np.uint32)
    src_off = np.zeros(n, np.uint64)
    if n:
        src_off[1:] = np.cumsum(src_len[:-1].astype(np.uint64))
    cap = np.array(caps, np.uint32)
    dst_off = np.zeros(n, np.uint64)
    if n:
        dst_off[1:] = np.cumsum(cap[:-1].astype(np.uint64))
    dev = torch.device("cuda")
    src = torch.from_numpy(np.frombuffer(b"".join(payloads) + b"\0", np.uint8).copy()).to(dev)
    dst = torch.zeros(int(cap.astype(np.uint64).sum()) + 1, dtype=torch.uint8, device=dev)
    t = {k: torch.from_numpy(v.view(np.int64 if v.dtype == np.uint64 else np.int32)).to(dev)
         for k, v in (("src_off", src_off), ("src_len", src_len), ("dst_off", dst_off), ("cap", cap))}
    out_len = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    status = torch.full((max(n, 1),), -1, dtype=torch.int32, device=dev)
    s = stream if stream is not None else torch.cuda.current_stream()
    L.check(L.lib().pvvc_zstd_inflate_batch(n, C.c_void_p(src.data_ptr()), C.c_void_p(t["src_off"].data_ptr()),
                                            C.c_void_p(t["src_len"].data_ptr()), C.c_void_p(dst.data_ptr()),
                                            C.c_void_p(t["dst_off"].data_ptr()), C.c_void_p(t["cap"].data_ptr()),
                                            C.c_void_p(out_len.data_ptr()), C.c_void_p(status.data_ptr()),
                                            C.c_void_p(s.cuda_stream)), "zstd_inflate_batch")
    torch.cuda.synchronize()
    d = dst.cpu().numpy()
    ol = out_len.cpu().numpy()[:n]
    st = status.cpu().numpy()[:n]
    outs = [d[int(dst_off[j]):int(dst_off[j]) + int(ol[j])].tobytes() if st[j] == 0 else b"" for j in range(n)]
    return outs, [int(x) for x in st]
