"""pvvc_fitting_clouds (PatchFitting::Compute with direct clustering,
src/patch/patch_fitting.cc:92-381) on the GPU: every GoP of a batch equal bit
for bit to the reference's fitting cloud in the golden fixture -- including
GoPs whose k-means empties clusters and redraws them from rand(), which needs
the cells' draws to be re-placed over several device rounds -- and to the
oracle on registered config-1 patch GoPs with other seeds."""
import numpy as np
import pytest

from test_fitting import fitting_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fitter(pvvc_lib):
    import torch
    assert torch.cuda.is_available()
    from pvvc.fitting import Fitter
    return Fitter()


def test_fitting_batch_matches_reference_fixture(fitter):
    cases = list(fitting_cases())
    clouds, st = fitter.fit([c[0] for c in cases], seeds=[c[1] for c in cases])
    for g, (got, (_, _, want)) in enumerate(zip(clouds, cases)):
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (g, got.shape, want.shape)
    assert st["empty_redraws"] > 0 and st["device_rounds"] > 1
    # each GoP alone gives the same cloud as in the batch
    for g in (0, 6, 8):
        one, _ = fitter.fit([cases[g][0]], seeds=[cases[g][1]])
        assert np.array_equal(one[0].view(np.uint32), clouds[g].view(np.uint32))


def test_fitting_registered_gops_vs_oracle(fitter, oracle, pvvc_lib):
    from pvvc import encode_flow as ef
    s = pvvc_lib.Synth(pvvc_lib.config("gof8", seed=4))
    src = ef.GopSource(s, 0, seed=2)
    gops = []
    for p in range(10):
        pats = [src.fit[p]]
        for f in range(1, src.nframes):
            inv = np.linalg.inv(src.true_mv[p][f].astype(np.float64))
            pats.append((src.frames[p][f][0].astype(np.float64) @ inv[:3, :3].T + inv[:3, 3]).astype(np.float32))
        gops.append(pats)
    seeds = list(range(5, 15))
    clouds, st = fitter.fit(gops, seeds=seeds)
    assert st["cells"] > 10
    for g in range(10):
        want, _ = oracle.fitting_cloud(gops[g], seed=seeds[g])
        assert np.array_equal(clouds[g].view(np.uint32), want.view(np.uint32)), g
