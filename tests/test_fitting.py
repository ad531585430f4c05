"""The GoP encoder's fitting cloud (PatchFitting::Compute with direct
clustering, src/patch/patch_fitting.cc:92-381) in the oracle: equal bit for
bit to the reference's own outputs in the golden fixture (registered patch
GoPs, and GoPs of repeated points whose k-means redraws empty clusters from
rand()) and -- where the reference tree is present -- to the reference
compiled here."""
import os

import numpy as np

from conftest import GOLDEN


def fitting_cases():
    z = np.load(os.path.join(GOLDEN, "fitting.npz"))
    po, gp, fo = z["patch_off"], z["gop_patch"], z["fit_off"]
    for g in range(len(gp) - 1):
        pats = [z["xyz"][po[p]:po[p + 1]] for p in range(gp[g], gp[g + 1])]
        yield pats, int(z["seeds"][g]), z["fit"][fo[g]:fo[g + 1]]


def test_oracle_fitting_matches_reference_fixture(oracle):
    n = redraws = 0
    for pats, seed, want in fitting_cases():
        got, st = oracle.fitting_cloud(pats, seed=seed)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (n, got.shape, want.shape)
        redraws += st["empty_redraws"]
        n += 1
    assert n == 9 and redraws > 0


def test_oracle_fitting_matches_reference_build(oracle, reference, pvvc_lib):
    rng = np.random.default_rng(8)
    for t in range(6):
        base = rng.integers(0, 12, (int(rng.integers(10, 80)), 3)).astype(np.float32)
        pats = [base[rng.integers(0, base.shape[0], int(rng.integers(20, 120)))] + rng.normal(0, 0.2, (1, 3)).astype(np.float32)
                for _ in range(int(rng.integers(3, 8)))]
        for seed in (1, 99):
            got, _ = oracle.fitting_cloud(pats, seed=seed)
            want = reference.fitting_cloud(pats, seed=seed)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
