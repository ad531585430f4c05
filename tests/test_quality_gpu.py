"""pvvc_cloud_quality (common::MSE::Compute, src/registration/
registration_base.cc:160-223) on the GPU against the reference's own outputs
(golden fixture) and the oracle.  The neighbours are exact and tie-broken as
in the oracle, so only the sums differ: the GPU adds in double, the reference
and the oracle in float in point order -- hence a relative tolerance."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

RTOL_SMALL = 2e-5   # a few thousand float additions
RTOL_LARGE = 2e-4   # ~10^5 float additions


@pytest.fixture(scope="module")
def q(pvvc_lib):
    import torch
    assert torch.cuda.is_available()
    from pvvc.quality import Quality
    return Quality()


def test_quality_matches_reference_fixture(q):
    z = np.load(os.path.join(GOLDEN, "cloud_quality.npz"))
    ao, bo = z["a_off"], z["b_off"]
    for k in range(len(ao) - 1):
        a, ac = z["a"][ao[k]:ao[k + 1]], z["a_rgb"][ao[k]:ao[k + 1]]
        b, bc = z["b"][bo[k]:bo[k + 1]], z["b_rgb"][bo[k]:bo[k + 1]]
        got = q.mse(a, ac, b, bc)
        want = z["mse"][k]
        assert np.allclose(got, want, rtol=RTOL_SMALL, atol=1e-6), (k, got, want)


def test_quality_large_clouds_vs_oracle(q, oracle, pvvc_lib):
    """A synthetic frame (~100k points) against a moved, jittered, rounded
    and recoloured copy, and against a copy 40 voxels away (the nearest
    neighbours then lie many grid rings out)."""
    s = pvvc_lib.Synth(pvvc_lib.config("gof8", nframes=1, gof=1, seed=9))
    rng = np.random.default_rng(5)
    xs = [s.patch(0, p)[0] for p in range(s.patch_count(0))]
    a = np.concatenate(xs).astype(np.float32)
    ac = rng.integers(0, 256, a.shape).astype(np.uint8)
    keep = rng.random(a.shape[0]) > 0.1
    b = np.round(a[keep] + rng.normal(0, 0.6, (int(keep.sum()), 3))).astype(np.float32)
    bc = np.clip(np.round(ac[keep] + rng.normal(0, 5, b.shape)), 0, 255).astype(np.uint8)
    for bb in (b, b + np.float32(40.0)):
        got = q.mse(a, ac, bb, bc)
        want = oracle.cloud_quality(a, ac, bb, bc)
        assert np.allclose(got, want, rtol=RTOL_LARGE), (got, want)


def test_quality_empty_and_single(q, oracle):
    a = np.array([[1, 2, 3]], np.float32)
    ac = np.array([[10, 20, 30]], np.uint8)
    e = np.zeros((0, 3), np.float32)
    ec = np.zeros((0, 3), np.uint8)
    assert list(q.mse(e, ec, a, ac)) == [-1, 0, -1, 0, -1, 0, -1, 0]
    assert list(q.mse(a, ac, e, ec)) == [0, -1, 0, -1, 0, -1, 0, -1]
    b = np.array([[4, 6, 3], [1, 2, 3.5]], np.float32)
    bc = np.array([[0, 0, 0], [11, 20, 30]], np.uint8)
    assert np.allclose(q.mse(a, ac, b, bc), oracle.cloud_quality(a, ac, b, bc), rtol=1e-7)

