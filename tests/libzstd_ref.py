"""libzstd through ctypes: the library the reference calls for its zstd
payloads (ZstdEncoder / ZstdDecoder, src/common/entropy_codec.cc:304-360),
used by the tests as the zstd oracle and to make zstd frames."""
from __future__ import annotations

import ctypes as C
import ctypes.util

import numpy as np
import pytest

_Z = None


def z():
    """The loaded libzstd, or skip the test when this host has none."""
    global _Z
    if _Z is None:
        for name in ("libzstd.so.1", ctypes.util.find_library("zstd")):
            if not name:
                continue
            try:
                _Z = C.CDLL(name)
                break
            except OSError:
                pass
        if _Z is None:
            pytest.skip("libzstd is not installed on this host")
        _Z.ZSTD_compressBound.restype = C.c_size_t
        _Z.ZSTD_compressBound.argtypes = [C.c_size_t]
        _Z.ZSTD_compress.restype = C.c_size_t
        _Z.ZSTD_compress.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int]
        _Z.ZSTD_decompress.restype = C.c_size_t
        _Z.ZSTD_decompress.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]
        _Z.ZSTD_isError.restype = C.c_uint
        _Z.ZSTD_isError.argtypes = [C.c_size_t]
        _Z.ZSTD_getFrameContentSize.restype = C.c_ulonglong
        _Z.ZSTD_getFrameContentSize.argtypes = [C.c_void_p, C.c_size_t]
        _Z.ZSTD_createCCtx.restype = C.c_void_p
        _Z.ZSTD_freeCCtx.argtypes = [C.c_void_p]
        _Z.ZSTD_CCtx_setParameter.restype = C.c_size_t
        _Z.ZSTD_CCtx_setParameter.argtypes = [C.c_void_p, C.c_int, C.c_int]
        _Z.ZSTD_compress2.restype = C.c_size_t
        _Z.ZSTD_compress2.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]
        _Z.ZSTD_versionNumber.restype = C.c_uint
    return _Z


def version() -> int:
    return int(z().ZSTD_versionNumber())


def compress(data: bytes, level: int = 22, checksum: bool = False, content_size: bool = True) -> bytes:
    """ZSTD_compress (the reference's ZstdEncoder::Encode), or the advanced
    API when a checksum is wanted or the content size left out."""
    L = z()
    cap = L.ZSTD_compressBound(len(data))
    out = C.create_string_buffer(max(cap, 1))
    if not checksum and content_size:
        r = L.ZSTD_compress(out, cap, data, len(data), level)
    else:
        cc = L.ZSTD_createCCtx()
        L.ZSTD_CCtx_setParameter(cc, 100, level)  # ZSTD_c_compressionLevel
        L.ZSTD_CCtx_setParameter(cc, 201, int(checksum))  # ZSTD_c_checksumFlag
        L.ZSTD_CCtx_setParameter(cc, 200, int(content_size))  # ZSTD_c_contentSizeFlag
        r = L.ZSTD_compress2(cc, out, cap, data, len(data))
        L.ZSTD_freeCCtx(cc)
    assert not L.ZSTD_isError(r)
    return out.raw[:r]


def decompress(data: bytes, cap: int):
    """ZSTD_decompress(dst, cap, data): the bytes, or None on error."""
    L = z()
    out = C.create_string_buffer(max(cap, 1))
    r = L.ZSTD_decompress(out, cap, data, len(data))
    return None if L.ZSTD_isError(r) else out.raw[:r]


def content_size(data: bytes) -> int:
    return int(z().ZSTD_getFrameContentSize(data, len(data)))


def sample_payloads(rng: np.random.Generator, count: int, max_len: int = 20000) -> list[bytes]:
    """Byte strings of several kinds: random, runs, small alphabets, repeats
    at short offsets, arithmetic patterns, and skewed (RLGR-like) bytes."""
    out = []
    for i in range(count):
        n = int(rng.integers(0, max_len))
        kind = i % 6
        if kind == 0:
            b = rng.integers(0, 256, n, dtype=np.uint8)
        elif kind == 1:
            b = np.repeat(rng.integers(0, 256, n // 8 + 1, dtype=np.uint8), 8)[:n]
        elif kind == 2:
            b = rng.integers(0, 4, n, dtype=np.uint8)
        elif kind == 3:
            base = rng.integers(0, 256, 64, dtype=np.uint8)
            b = np.tile(base, n // 64 + 1)[:n].copy()
            flip = rng.random(n) < 0.05
            b[flip] = rng.integers(0, 256, int(flip.sum()), dtype=np.uint8)
        elif kind == 4:
            idx = np.arange(n, dtype=np.int64)
            b = ((idx * 7) ^ (idx >> 5)).astype(np.uint8)
        else:
            b = np.minimum(np.abs(rng.normal(0, 8, n)), 255).astype(np.uint8)
        out.append(b.tobytes())
    return out


def zstd_frame(frame: bytes, pvvc, level: int = 22) -> bytes:
    """A .frame with each payload zstd-compressed where that makes it smaller,
    and the slice type's zstd bit set, as GoPEncoding::Encode does
    (src/patch/GoP_encoding.cc:158-200)."""
    f = pvvc.parse_frame(frame)
    for i in range(f.n):
        g, c = bytes(f.geometry[i]), bytes(f.color[i])
        if g:
            zg = compress(g, level)
            if len(zg) < len(g):
                f.geometry[i] = zg
                f.type[i] |= 0x08
        if c:
            zc = compress(c, level)
            if len(zc) < len(c):
                f.color[i] = zc
                f.type[i] |= 0x10
    return pvvc.write_frame(f)
