"""The zstd decoder on the host (pvvc_zstd_inflate_host, the same code the
GPU kernel runs) against libzstd, the library the reference's ZstdDecoder
calls (src/common/entropy_codec.cc:341-360)."""
import numpy as np
import pytest

import libzstd_ref as zr
from conftest import golden_frames


def _inflate(pvvc_lib, data, cap):
    try:
        return pvvc_lib.zstd.inflate_host(data, cap)
    except pvvc_lib.PvvcError:
        return None


@pytest.mark.parametrize("level", [1, 3, 19, 22, -5])
def test_host_inflate_matches_libzstd(pvvc_lib, level):
    rng = np.random.default_rng(100 + level)
    for data in zr.sample_payloads(rng, 24) + [b"", b"x", bytes(300_000)]:
        c = zr.compress(data, level)
        assert _inflate(pvvc_lib, c, len(data)) == data
        assert zr.decompress(c, len(data)) == data


def test_host_inflate_multi_block_and_large(pvvc_lib):
    rng = np.random.default_rng(7)
    big = zr.sample_payloads(rng, 6, max_len=600_000)
    for data in big:
        c = zr.compress(data, 3)
        assert _inflate(pvvc_lib, c, len(data)) == data


def test_host_inflate_reference_golden_payloads(pvvc_lib):
    """The reference encoder's own zstd payloads (level 22, geometry and
    colour), from the golden .frame files."""
    seen = 0
    for b in golden_frames("zstd"):
        f = pvvc_lib.parse_frame(b)
        for i in range(f.n):
            for bit, payload in ((0x08, f.geometry[i]), (0x10, f.color[i])):
                if f.type[i] & bit and len(payload):
                    cap = zr.content_size(payload)
                    assert pvvc_lib.zstd.content_size(payload) == cap
                    assert _inflate(pvvc_lib, payload, cap) == zr.decompress(payload, cap)
                    seen += 1
    assert seen > 0


def test_host_inflate_frames_checksums_and_skippable(pvvc_lib):
    a, b = b"abc" * 5000, bytes(range(256)) * 40
    ca = zr.compress(a, 19, checksum=True)
    cb = zr.compress(b, 1, content_size=False)
    skip = (0x184D2A53).to_bytes(4, "little") + (5).to_bytes(4, "little") + b"12345"
    stream = ca + skip + cb + skip
    cap = len(a) + len(b)
    assert _inflate(pvvc_lib, stream, cap) == zr.decompress(stream, cap) == a + b
    # a wrong checksum, too little room, trailing bytes: both reject
    bad_sum = ca[:-1] + bytes([ca[-1] ^ 1])
    for data, c in ((bad_sum, len(a)), (stream, cap - 1), (ca + b"\0\0", len(a))):
        assert zr.decompress(data, c) is None
        assert _inflate(pvvc_lib, data, c) is None
    assert pvvc_lib.zstd.content_size(cb) == pvvc_lib.zstd.UNKNOWN == zr.content_size(cb)
    assert pvvc_lib.zstd.content_size(skip) == 0 == zr.content_size(skip)


def test_host_content_size_field_widths(pvvc_lib):
    for n in (0, 1, 255, 256, 300, 65535 + 256, 65536 + 256, 100_000):
        c = zr.compress(bytes(n), 3)
        assert pvvc_lib.zstd.content_size(c) == zr.content_size(c) == n
    with pytest.raises(pvvc_lib.PvvcError):
        pvvc_lib.zstd.content_size(b"\x28\xb5\x2f")


def test_host_inflate_corrupt_never_accepts_what_libzstd_rejects(pvvc_lib):
    """Single-byte corruptions and truncations: whenever both decoders accept,
    the bytes agree; the GPU decoder never accepts a frame libzstd rejects."""
    rng = np.random.default_rng(5)
    lib_only = 0
    for data in zr.sample_payloads(rng, 60, max_len=8000):
        c = bytearray(zr.compress(data, int(rng.choice([1, 3, 19]))))
        if len(c) < 8:
            continue
        for _ in range(4):
            d = bytearray(c)
            d[int(rng.integers(0, len(d)))] ^= int(rng.integers(1, 256))
            want, got = zr.decompress(bytes(d), len(data)), _inflate(pvvc_lib, bytes(d), len(data))
            if want is None:
                assert got is None
            elif got is None:
                lib_only += 1  # a Huffman stream that does not end on its first bit
            else:
                assert got == want
        t = bytes(c[:int(rng.integers(0, len(c)))])  # truncated (an empty input decodes to nothing in both)
        assert zr.decompress(t, len(data)) == _inflate(pvvc_lib, t, len(data))
    assert lib_only < 60
