"""GPU colour interpolation (pvvc_knn_colors_batch) against the oracle, bit
for bit: the GoP encoder's k-NN colour interpolation
(src/patch/GoP_encoding.cc:73-95,131-150) over seeded patch pairs with
voxel coordinates (many equal distances), k from 1 to 16, frame-0 residuals,
patches smaller than k, and an empty patch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


def _gop_pairs(pvvc_lib, nframes, seed):
    """Fitting clouds (patch geometry of a synthetic GoP) and, per frame, a
    source patch: the cloud moved by up to a voxel, 10% of points dropped,
    integer coordinates, RGB from the frame's YUV."""
    s = pvvc_lib.Synth(pvvc_lib.config("gof8", nframes=nframes, gof=nframes, seed=seed))
    rng = np.random.default_rng(seed)
    queries, query_of, sources, rgbs, base = [], [], [], [], []
    for p in range(s.patch_count(0)):
        xyz, yuv = s.patch(0, p)[:2]
        qi = len(queries)
        queries.append(xyz.astype(np.float32))
        first = len(sources)
        for f in range(nframes):
            keep = rng.random(xyz.shape[0]) > 0.1
            keep[0] = True
            src = np.round(xyz[keep] + rng.integers(-1, 2, (int(keep.sum()), 3))).astype(np.float32)
            rgb = np.clip(yuv[f][keep] + 128 if f else yuv[0][keep], 0, 255).astype(np.uint8)
            query_of.append(qi)
            sources.append(src)
            rgbs.append(rgb)
            base.append(-1 if f == 0 else first)
    return queries, query_of, sources, rgbs, base


@pytest.mark.parametrize("k", [1, 4, 10, 16])
def test_knn_colors_gpu_equal_oracle(pvvc_lib, oracle, torch, k):
    from pvvc.icp import KnnColorBatch
    queries, query_of, sources, rgbs, base = _gop_pairs(pvvc_lib, 3, 31 + k)
    b = KnnColorBatch(queries, query_of, sources, rgbs, k=k)
    b.run()
    got, st = b.results()
    assert (st == 0).all()
    for p in range(len(sources)):
        want = oracle.knn_colors(queries[query_of[p]], sources[p], rgbs[p], k)
        assert np.array_equal(got[p].view(np.uint32), want.view(np.uint32)), (p, k)


def test_knn_colors_gpu_residuals_against_frame0(pvvc_lib, oracle, torch):
    from pvvc.icp import KnnColorBatch
    queries, query_of, sources, rgbs, base = _gop_pairs(pvvc_lib, 4, 7)
    absolute = KnnColorBatch(queries, query_of, sources, rgbs, k=10)
    absolute.run()
    a, st_a = absolute.results()
    resid = KnnColorBatch(queries, query_of, sources, rgbs, k=10, base=base)
    resid.run()
    r, st_r = resid.results()
    assert (st_a == 0).all() and (st_r == 0).all()
    for p, bp in enumerate(base):
        want = a[p] if bp < 0 else (a[p] - a[bp]).astype(np.float32)  # ColorYUV::operator-= in float
        assert np.array_equal(r[p].view(np.uint32), want.view(np.uint32)), p


def test_knn_colors_gpu_small_empty_and_bad_arguments(pvvc_lib, oracle, torch):
    from pvvc.icp import KnnColorBatch
    rng = np.random.default_rng(5)
    q = rng.integers(0, 20, (300, 3)).astype(np.float32)
    small = rng.integers(0, 20, (3, 3)).astype(np.float32)   # fewer points than k
    one = q[:1].copy()
    empty = np.zeros((0, 3), np.float32)
    c3 = rng.integers(0, 256, (3, 3)).astype(np.uint8)
    c1 = rng.integers(0, 256, (1, 3)).astype(np.uint8)
    b = KnnColorBatch([q], [0, 0, 0], [small, empty, one], [c3, np.zeros((0, 3), np.uint8), c1], k=16,
                      base=[-1, -1, 0])
    b.run()
    got, st = b.results()
    assert st[0] == 0 and st[1] == 1 and st[2] == 0
    assert np.array_equal(got[0].view(np.uint32), oracle.knn_colors(q, small, c3, 16).view(np.uint32))
    assert (got[1] == 0).all()
    want2 = (oracle.knn_colors(q, one, c1, 16) - oracle.knn_colors(q, small, c3, 16)).astype(np.float32)
    assert np.array_equal(got[2].view(np.uint32), want2.view(np.uint32))
    # a base that has a base of its own is rejected
    bad = KnnColorBatch([q], [0, 0, 0], [small, one, small], [c3, c1, c3], k=4, base=[-1, 0, 1])
    bad.run()
    _, st = bad.results()
    assert st[2] == 1
    for k in (0, 17):
        with pytest.raises(pvvc_lib.PvvcError):
            KnnColorBatch([q], [0], [small], [c3], k=k).run()


def test_knn_colors_gpu_equal_reference_gop_encoding(pvvc_lib, torch):
    """The GPU's colours equal the reference GoPEncoding::Encode's
    patch_colors_ (golden fixture), residuals included, bit for bit."""
    from pvvc.icp import KnnColorBatch
    from test_knn_colors import _golden
    k, _, pats = _golden()
    queries, query_of, sources, rgbs, base = [], [], [], [], []
    for p, (fit, srcs, rg, _, _, _) in enumerate(pats):
        first = len(sources)
        for f, (s, c) in enumerate(zip(srcs, rg)):
            query_of.append(p)
            sources.append(s)
            rgbs.append(c)
            base.append(-1 if f == 0 else first)
        queries.append(fit)
    b = KnnColorBatch(queries, query_of, sources, rgbs, k=k, base=base)
    b.run()
    got, st = b.results()
    assert (st == 0).all()
    i = 0
    for fit, srcs, _, cols, _, _ in pats:
        for f in range(len(srcs)):
            assert np.array_equal(got[i].view(np.uint32), cols[f].view(np.uint32)), (i, f)
            i += 1
