"""Host-side product code on CPU: the RLGR codec and GoP encoder of the
library against the reference's golden bytes and the oracle, the .frame
layout, the synthetic generator, and the C ABI's exported symbols."""
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden_frames


def _rlgr_golden():
    z = np.load(os.path.join(GOLDEN, "rlgr.npz"))
    so, bo = z["sym_off"], z["byte_off"]
    for i in range(len(so) - 1):
        yield z["symbols"][so[i]:so[i + 1]], z["bytes"][bo[i]:bo[i + 1]].tobytes(), z["decoded"][so[i]:so[i + 1]]


def test_library_exports_every_declared_symbol(pvvc_lib):
    import ctypes
    lib = ctypes.CDLL(pvvc_lib.LIB_PATH)
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(pvvc_[a-z0-9_]+)\s*\(", src))
    assert names, "no declarations found"
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_host_rlgr_encoder_matches_reference_bytes(pvvc_lib):
    for sym, enc, dec in _rlgr_golden():
        assert pvvc_lib.rlgr_encode(sym) == enc
        assert np.array_equal(pvvc_lib.rlgr_decode(enc, sym.size), dec)


def test_host_rlgr_decode_truncated(pvvc_lib):
    sym, enc, _ = next(iter(_rlgr_golden()))
    with pytest.raises(pvvc_lib.PvvcError) as e:
        pvvc_lib.rlgr_decode(enc[: len(enc) // 3], sym.size)
    assert e.value.status == 2


def test_host_rlgr_empty_and_single(pvvc_lib, oracle):
    for s in ([], [0], [5], [-1], [0] * 1000, [0] * 999 + [-1]):
        s = np.array(s, np.int64)
        e = pvvc_lib.rlgr_encode(s)
        assert e == oracle.rlgr_encode(s)
        if s.size:
            assert np.array_equal(pvvc_lib.rlgr_decode(e, s.size), s)


def test_gop_encoder_matches_oracle(pvvc_lib, oracle):
    s = pvvc_lib.Synth(pvvc_lib.config("gof8", nframes=3, gof=3, seed=5))
    for p in range(0, s.patch_count(0), 7):
        xyz, yuv, mv = s.patch(0, p)
        qps = [4, 16, 32]
        g1, n1, c1 = pvvc_lib.encode_patch_gop(xyz, yuv, qps)
        g2, n2, c2, _ = oracle.encode_patch(xyz, list(yuv), qps)
        assert g1 == g2 and n1 == n2 and c1 == c2


def test_gop_encoder_edge_patches(pvvc_lib, oracle):
    rng = np.random.default_rng(1)
    cases = [np.array([[3.0, 4.0, 5.0]]), np.array([[0, 0, 0], [1000, 0, 0]], float),
             rng.integers(0, 4, (200, 3)).astype(float),            # many points per voxel
             rng.uniform(-50, 50, (500, 3)),                          # non-integer, negative
             np.stack(np.meshgrid(*[np.arange(16)] * 3, indexing="ij"), -1).reshape(-1, 3).astype(float)]
    for xyz in cases:
        xyz = xyz.astype(np.float32)
        yuv = rng.uniform(0, 255, (2,) + xyz.shape).astype(np.float32)
        g1, n1, c1 = pvvc_lib.encode_patch_gop(xyz, yuv, [8, 8])
        g2, n2, c2, _ = oracle.encode_patch(xyz, list(yuv), [8, 8])
        assert g1 == g2 and n1 == n2 and c1 == c2


def test_frame_layout_of_reference_files(pvvc_lib):
    for b in golden_frames("raw") + golden_frames("zstd"):
        fr = pvvc_lib.parse_frame(b)
        assert fr.n == 8
        assert pvvc_lib.write_frame(fr) == b     # byte-identical round trip
    f0 = pvvc_lib.parse_frame(golden_frames("zstd")[0])
    assert (f0.type & 0x08).any()                # the fixture exercises zstd geometry


def test_synth_is_deterministic_and_sized(pvvc_lib):
    a = pvvc_lib.Synth(pvvc_lib.config("gof8"))
    b = pvvc_lib.Synth(pvvc_lib.config("gof8"))
    assert a.patch_count(0) == b.patch_count(0)
    n = 0
    for p in range(a.patch_count(0)):
        xa, ya, ma = a.patch(0, p)
        xb, yb, mb = b.patch(0, p)
        assert np.array_equal(xa, xb) and np.array_equal(ya, yb) and np.array_equal(ma, mb)
        n += xa.shape[0]
        assert 800 <= xa.shape[0] <= 2500 + 800
    assert 70_000 < n < 140_000
    fa, fb = a.frames(), b.frames()
    assert fa == fb and len(fa) == 8


def test_invalid_launch_shape_is_rejected_before_any_device_work(pvvc_lib):
    s = pvvc_lib.Synth(pvvc_lib.config("tiny", seed=3))
    batch = pvvc_lib.pack_frames([pvvc_lib.parse_frame(b) for b in s.frames()[:1]])
    for t in [(5, 4, 128, 0, 0, 0), (1, 33, 128, 0, 0, 0), (1, 4, 96, 0, 0, 0), (-1, 4, 128, 0, 0, 0),
              (1, 4, 128, 153, 0, 0), (1, 4, 128, -2, 0, 0), (1, 4, 128, 0, 91, 0), (1, 4, 128, 0, -2, 0),
              (1, 4, 128, 0, 0, 12)]:
        with pytest.raises(pvvc_lib.PvvcError) as e:
            pvvc_lib.Plan(batch, tune=t)
        assert e.value.status == 1
