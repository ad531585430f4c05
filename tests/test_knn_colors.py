"""Colour interpolation of the GoP encoder (GoPEncoding::Interpolation and
its k-NN loop, src/patch/GoP_encoding.cc:73-95,131-150) in the oracle: the
grid search returns the brute-force neighbours, and the arithmetic equals an
independent float32 restatement, bit for bit.  PCL's k-d tree is not
available here, so the neighbour order among equal distances (lower source
index first) is this project's rule; parity against PCL is unpinned."""
import numpy as np
import pytest


def _restated(q, src, rgb, k):
    """The reference's statements in numpy float32, one query at a time."""
    f = np.float32
    out = np.zeros((q.shape[0], 3), np.float32)
    for t in range(q.shape[0]):
        d = src - q[t]
        dd = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        order = np.lexsort((np.arange(src.shape[0]), dd))[:min(k, src.shape[0])]
        w = [f(1) / max(dd[j], f(1e-6)) for j in order]
        s = f(0)
        for x in w:
            s = f(s + x)
        w = [f(x / s) for x in w]
        r = g = b = f(0)
        for x, j in zip(w, order):
            r = f(r + f(x * f(rgb[j, 0])))
            g = f(g + f(x * f(rgb[j, 1])))
            b = f(b + f(x * f(rgb[j, 2])))
        out[t, 0] = f(f(f(r * f(0.299)) + f(g * f(0.587))) + f(b * f(0.114)))
        out[t, 1] = f(f(f(f(r * f(-0.168736)) - f(g * f(0.331264))) + f(b * f(0.5))) + f(128))
        out[t, 2] = f(f(f(f(r * f(0.5)) - f(g * f(0.418688))) - f(b * f(0.081312))) + f(128))
    return out


@pytest.mark.parametrize("voxel", [True, False])
def test_oracle_knn_colors_grid_equals_brute_force_and_restatement(oracle, voxel):
    rng = np.random.default_rng(11 if voxel else 12)
    for n in (3, 40, 350):
        if voxel:  # integer clouds: many equal distances
            src = rng.integers(0, 12, (n, 3)).astype(np.float32)
            q = rng.integers(-2, 14, (150, 3)).astype(np.float32)
        else:
            src = rng.normal(0, 5, (n, 3)).astype(np.float32)
            q = rng.normal(0, 5, (150, 3)).astype(np.float32)
        rgb = rng.integers(0, 256, (n, 3)).astype(np.uint8)
        for k in (1, 4, 10, 16):
            a = oracle.knn_colors(q, src, rgb, k, brute=True)
            b = oracle.knn_colors(q, src, rgb, k, brute=False)
            c = _restated(q, src, rgb, k)
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (n, k)
            assert np.array_equal(a.view(np.uint32), c.view(np.uint32)), (n, k)


def test_oracle_knn_colors_known_answers(oracle):
    src = np.array([[0, 0, 0], [1, 0, 0], [5, 5, 5]], np.float32)
    rgb = np.array([[255, 0, 0], [0, 255, 0], [0, 0, 255]], np.uint8)
    # k=1 on a source point: its own colour (d clamped to 1e-6, weight 1)
    y = oracle.knn_colors(src[:1], src, rgb, 1)[0]
    f = np.float32
    assert y[0] == f(f(f(f(255) * f(0.299)) + f(0) * f(0.587)) + f(0) * f(0.114))
    # midway between two points at equal distance: equal weights
    y = oracle.knn_colors(np.array([[0.5, 0, 0]], np.float32), src, rgb, 2)[0]
    r = g = f(f(1) / f(0.25)) / f(f(f(1) / f(0.25)) + f(f(1) / f(0.25)))
    assert y[0] == f(f(f(f(r * f(255)) * f(0.299)) + f(f(g * f(255)) * f(0.587))) + f(0) * f(0.114))
    # k larger than the patch: every point, no error
    assert np.isfinite(oracle.knn_colors(src, src, rgb, 16)).all()
    with pytest.raises(RuntimeError):
        oracle.knn_colors(src, src[:0], rgb[:0], 4)


def _golden():
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "gop_encode.npz"))
    nf = int(z["nframes"])
    fo, so, go, po = z["fit_off"], z["src_off"], z["geo_off"], z["pay_off"]
    pats = []
    for p in range(len(fo) - 1):
        fit = z["fit"][fo[p]:fo[p + 1]].astype(np.float32)
        n = fit.shape[0]
        srcs = [z["src"][so[p * nf + f]:so[p * nf + f + 1]].astype(np.float32) for f in range(nf)]
        rgbs = [z["rgb"][so[p * nf + f]:so[p * nf + f + 1]].astype(np.uint8) for f in range(nf)]
        base = int(sum(fo[q + 1] - fo[q] for q in range(p))) * nf
        cols = z["colors"][base:base + nf * n].reshape(nf, n, 3).astype(np.float32)
        geo = z["geo"][go[p]:go[p + 1]].tobytes()
        pays = [z["pay"][po[p * nf + f]:po[p * nf + f + 1]].tobytes() for f in range(nf)]
        pats.append((fit, srcs, rgbs, cols, geo, pays))
    return int(z["k"]), [int(z["qp_i"])] + [int(z["qp_p"])] * (nf - 1), pats


def test_oracle_and_host_encoder_match_reference_gop_encoding(oracle, pvvc_lib):
    """Pinned against the reference's own GoPEncoding::Encode (golden
    fixture from tests/golden/make_golden.py, its k-d tree the shim's exact
    search): the interpolated colours bit for bit, and the host encoder's
    geometry and colour payloads byte for byte."""
    k, qps, pats = _golden()
    for fit, srcs, rgbs, cols, geo, pays in pats:
        mine = np.stack([oracle.knn_colors(fit, s, c, k) for s, c in zip(srcs, rgbs)])
        mine[1:] = (mine[1:] - mine[0]).astype(np.float32)  # ColorYUV::operator-= (GoP_encoding.cc:144-148)
        assert np.array_equal(mine.view(np.uint32), cols.view(np.uint32))
        g, _, cp = pvvc_lib.encode_patch_gop(fit, mine, qps)
        assert g == geo
        assert all(a == b for a, b in zip(cp, pays))
