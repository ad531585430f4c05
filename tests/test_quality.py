"""common::MSE::Compute (src/registration/registration_base.cc:160-223) in the
oracle: equal to the reference's own outputs in the golden fixture and --
where the reference tree is present -- to the reference compiled here, and
its grid search equal to its brute-force search."""
import os

import numpy as np

from conftest import GOLDEN


def _pairs():
    z = np.load(os.path.join(GOLDEN, "cloud_quality.npz"))
    ao, bo = z["a_off"], z["b_off"]
    for k in range(len(ao) - 1):
        yield (z["a"][ao[k]:ao[k + 1]], z["a_rgb"][ao[k]:ao[k + 1]], z["b"][bo[k]:bo[k + 1]], z["b_rgb"][bo[k]:bo[k + 1]],
               z["mse"][k])


def test_oracle_quality_matches_reference_fixture(oracle):
    n = 0
    for a, ac, b, bc, want in _pairs():
        got = oracle.cloud_quality(a, ac, b, bc)
        assert np.array_equal(got.astype(np.float32), want.astype(np.float32)), (got, want)
        assert np.array_equal(oracle.cloud_quality(a, ac, b, bc, brute=True), got)
        n += 1
    assert n == 6


def test_oracle_quality_empty_clouds(oracle):
    a = np.zeros((5, 3), np.float32)
    c = np.zeros((5, 3), np.uint8)
    e = np.zeros((0, 3), np.float32)
    assert list(oracle.cloud_quality(e, e.astype(np.uint8), a, c)) == [-1, 0, -1, 0, -1, 0, -1, 0]
    assert list(oracle.cloud_quality(a, c, e, e.astype(np.uint8))) == [0, -1, 0, -1, 0, -1, 0, -1]


def test_oracle_quality_matches_reference_build(oracle, reference):
    rng = np.random.default_rng(3)
    for t in range(4):
        na, nb = int(rng.integers(1, 2500)), int(rng.integers(1, 2500))
        a = (rng.integers(0, 50, (na, 3)) + 0.5 * (rng.random((na, 3)) < 0.3)).astype(np.float32)
        b = rng.integers(0, 50, (nb, 3)).astype(np.float32)
        ac = rng.integers(0, 256, (na, 3)).astype(np.uint8)
        bc = rng.integers(0, 256, (nb, 3)).astype(np.uint8)
        assert np.array_equal(oracle.cloud_quality(a, ac, b, bc), reference.mse_compute(a, ac, b, bc))


def test_psnr_formula(pvvc_lib):
    from pvvc.quality import psnr
    m = np.array([0.5, 0.25, 16.0, 20.0, 4.0, 2.0, 1.0, 3.0])
    p = psnr(m)
    assert abs(p["geo"] - 10 * np.log10(1024 ** 2 / 0.5)) < 1e-12
    assert abs(p["y"] - 10 * np.log10(256 ** 2 / 20.0)) < 1e-12
