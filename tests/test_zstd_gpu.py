"""The GPU zstd inflater (pvvc_zstd_inflate_batch, one warp per payload)
against libzstd, the library the reference's ZstdDecoder calls
(src/common/entropy_codec.cc:341-360)."""
import numpy as np
import pytest

import libzstd_ref as zr
from conftest import golden_frames

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def test_gpu_inflate_matches_libzstd(pvvc_lib, torch):
    rng = np.random.default_rng(11)
    datas = zr.sample_payloads(rng, 300) + zr.sample_payloads(rng, 6, max_len=400_000) + [b"", b"q", bytes(200_000)]
    levels = [1, 3, 9, 19, 22, -5]
    comp = [zr.compress(d, levels[i % len(levels)]) for i, d in enumerate(datas)]
    outs, st = pvvc_lib.zstd.inflate_device(comp, [len(d) for d in datas])
    assert st == [0] * len(datas)
    for o, d in zip(outs, datas):
        assert o == d


def test_gpu_inflate_reference_golden_payloads(pvvc_lib, torch):
    payloads = []
    for b in golden_frames("zstd"):
        f = pvvc_lib.parse_frame(b)
        for i in range(f.n):
            for bit, p in ((0x08, f.geometry[i]), (0x10, f.color[i])):
                if f.type[i] & bit and len(p):
                    payloads.append(bytes(p))
    assert payloads
    caps = [zr.content_size(p) for p in payloads]
    outs, st = pvvc_lib.zstd.inflate_device(payloads, caps)
    assert st == [0] * len(payloads)
    assert outs == [zr.decompress(p, c) for p, c in zip(payloads, caps)]


def test_gpu_inflate_frames_checksums_corrupt(pvvc_lib, torch):
    rng = np.random.default_rng(12)
    a, b = b"abc" * 5000, bytes(range(256)) * 40
    ca, cb = zr.compress(a, 19, checksum=True), zr.compress(b, 1, content_size=False)
    skip = (0x184D2A5F).to_bytes(4, "little") + (3).to_bytes(4, "little") + b"xyz"
    jobs = [(ca + skip + cb, len(a) + len(b)), (ca[:-1] + bytes([ca[-1] ^ 1]), len(a)), (ca + skip + cb, len(a) + len(b) - 1),
            (ca + b"\0", len(a)), (b"", 0)]
    for d in zr.sample_payloads(rng, 40, max_len=6000):
        c = bytearray(zr.compress(d, 3))
        if len(c) > 8:
            c[int(rng.integers(0, len(c)))] ^= int(rng.integers(1, 256))
        jobs.append((bytes(c), len(d)))
    outs, st = pvvc_lib.zstd.inflate_device([j[0] for j in jobs], [j[1] for j in jobs])
    for (data, cap), o, s in zip(jobs, outs, st):
        want, host = zr.decompress(data, cap), None
        try:
            host = pvvc_lib.zstd.inflate_host(data, cap)
        except pvvc_lib.PvvcError:
            pass
        assert (s == 0) == (host is not None)  # the device and host builds decide alike
        if s == 0:
            assert o == host == want
        if want is None:
            assert s != 0
    assert st[0] == 0 and outs[0] == a + b
    assert st[1] != 0 and st[2] != 0 and st[3] != 0


def test_gpu_inflate_no_jobs_and_bad_args(pvvc_lib, torch):
    L = pvvc_lib.lib()
    assert L.pvvc_zstd_inflate_batch(0, None, None, None, None, None, None, None, None, None) == 0
    assert L.pvvc_zstd_inflate_batch(-1, None, None, None, None, None, None, None, None, None) != 0
    assert L.pvvc_zstd_inflate_batch(1, None, None, None, None, None, None, None, None, None) != 0
