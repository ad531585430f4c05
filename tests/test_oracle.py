"""The oracle (CPU restatement) against the reference's own outputs: the
golden fixtures generated by the reference's code, and -- where the reference
tree is present -- the reference compiled here."""
import numpy as np
import pytest

from conftest import GOLDEN, golden_expected, golden_frames, rgb_matches

import os


def _rlgr_golden():
    z = np.load(os.path.join(GOLDEN, "rlgr.npz"))
    so, bo = z["sym_off"], z["byte_off"]
    for i in range(len(so) - 1):
        yield z["symbols"][so[i]:so[i + 1]], z["bytes"][bo[i]:bo[i + 1]].tobytes(), z["decoded"][so[i]:so[i + 1]], int(z["kinds"][i])


def test_oracle_rlgr_matches_reference_bytes(oracle):
    n = 0
    for sym, enc, dec, kind in _rlgr_golden():
        assert oracle.rlgr_encode(sym) == enc
        assert np.array_equal(oracle.rlgr_decode(enc, sym.size), dec)
        if kind != 6:  # below 2^32 the code is lossless
            assert np.array_equal(dec, sym)
        n += 1
    assert n == 34


def test_oracle_rlgr_truncated_stream_reports_overrun(oracle):
    sym, enc, _, _ = next(iter(_rlgr_golden()))
    with pytest.raises(ValueError):
        oracle.rlgr_decode(enc[: len(enc) // 2], sym.size)


def test_oracle_decodes_golden_gop(pvvc_lib, oracle):
    exp = golden_expected()
    decs = [oracle.decoder() for _ in range(8)]
    for f, b in enumerate(golden_frames("raw")):
        fr = pvvc_lib.parse_frame(b)
        xyz, rgb, st = oracle.decode_frame(decs, fr)
        assert (st == 0).all()
        assert np.array_equal(xyz.view(np.uint32), exp[f"xyz_{f}"].view(np.uint32))
        # colours: equal to the reference wherever its uint8 cast is defined
        yuv = np.concatenate([d.get_patch()[1] for d in decs])
        assert rgb_matches(rgb, exp[f"rgb_{f}"], yuv).all()


def test_oracle_predictive_without_intra_is_rejected(pvvc_lib, oracle):
    fr = pvvc_lib.parse_frame(golden_frames("raw")[1])
    d = oracle.decoder()
    assert d.set_slice(int(fr.type[0]), int(fr.size[0]), int(fr.qp[0]), b"", fr.color[0]) == 5  # NO_REFERENCE


def test_oracle_encoder_matches_reference(pvvc_lib, oracle, reference):
    from oracle import quantise
    s = pvvc_lib.Synth(pvvc_lib.config("tiny", seed=3))
    for p in range(s.patch_count(0)):
        xyz, yuv, mv = s.patch(0, p)
        qps = [8] * yuv.shape[0]
        g1, n1, c1, k1 = oracle.encode_patch(xyz, list(yuv), qps)
        g2, n2, c2, k2 = reference.encode_patch(xyz, list(yuv), qps, quantise)
        assert g1 == g2 and n1 == n2 and c1 == c2
        for a, b in zip(k1, k2):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_oracle_decoder_matches_reference_on_random_patches(oracle, reference):
    from oracle import quantise
    rng = np.random.default_rng(11)
    for t in range(6):
        n = int(rng.integers(1, 1500))
        xyz = rng.integers(0, int(rng.integers(2, 150)), (n, 3)).astype(np.float32)
        yuv0 = rng.uniform(16, 235, (n, 3)).astype(np.float32)
        yuv1 = rng.normal(0, 20, (n, 3)).astype(np.float32)
        g, nl, cols, _ = reference.encode_patch(xyz, [yuv0, yuv1], [4, 4], quantise)
        do, dr = oracle.decoder(), reference.decoder()
        for f, typ in enumerate((1, 3)):
            assert do.set_slice(typ, nl, 4, g if f == 0 else b"", cols[f]) == 0
            assert dr.set_slice(typ, nl, 4, g if f == 0 else b"", cols[f]) == 0
            xo, yo, ro = do.get_patch()
            xr, rr = dr.get_patch(nl)
            assert np.array_equal(xo, xr)
            assert rgb_matches(ro, rr, yo).all()


def test_fp64_inverse_raht_restatement(pvvc_lib, oracle):
    """The FP64 restatement of the inverse RAHT (octree_base.cc:186-206 in
    double) against the FP32 one the reference (and the GPU, bit for bit)
    uses: on the reference-written golden GoP and on a synthetic GoP the FP32
    colours stay within 1e-3 of the FP64 ones, and RGB bytes differ by at most
    one.  An intra slice quantised with step 1 reproduces the encoder's leaf
    colours within the rounding of the symbols (|error| <= 0.5 per
    coefficient, orthonormal transform: at most 0.5 * sqrt(N) in norm)."""
    r = oracle.raht_fp64_error(golden_frames("raw"), pvvc_lib.parse_frame)
    assert r["values"] > 0 and r["yuv_max_abs"] < 1e-3 and r["rgb_max_abs"] <= 1
    s = pvvc_lib.Synth(pvvc_lib.config("gof8", seed=5))
    r = oracle.raht_fp64_error(s.frames(), pvvc_lib.parse_frame)
    assert r["yuv_max_abs"] < 1e-3 and r["rgb_max_abs"] <= 1 and r["rgb_frac_differing"] < 1e-3
    rng = np.random.default_rng(2)
    xyz = rng.integers(0, 40, (600, 3)).astype(np.float32)
    yuv = rng.uniform(16, 235, (600, 3)).astype(np.float32)
    geo, nl, leaf = pvvc_lib.patch_leaf_yuv(xyz, yuv[None])
    _, _, cols = pvvc_lib.encode_patch_gop(xyz, yuv[None], [1])
    d = oracle.decoder()
    d.enable_fp64()
    assert d.set_slice(1, nl, 1, geo, cols[0]) == 0
    err = d.get_yuv_fp64() - leaf[0].astype(np.float64)
    assert np.sqrt((err ** 2).sum(0)).max() <= 0.5 * np.sqrt(nl) + 1e-6
