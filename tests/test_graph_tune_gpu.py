"""Launch shapes, the autotuner and CUDA-graph replay of the decode: every
shape and the graph produce the same bytes as the default plan (which the
other decode tests pin to the oracle)."""
import numpy as np
import pytest

from test_decode_gpu import _dev, decode_batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


@pytest.fixture(scope="module")
def gop(pvvc_lib):
    s = pvvc_lib.Synth(pvvc_lib.config("gof8", seed=11))
    return pvvc_lib.pack_frames([pvvc_lib.parse_frame(b) for b in s.frames()])


# (group CTAs per SM, min group, RLGR block, long-slice CTAs (-1: no split), medium-tier % (-1: none),
#  slices per warp of the long launch)
TUNES = [
    (1, 1, 32, -1, -1, 32), (2, 2, 64, 1, -1, 8), (3, 4, 128, -1, 30, 16), (4, 16, 256, 4, 50, 16), (1, 32, 128, 32, 15, 32),
    (2, 8, 32, 2, 70, 8), (4, 3, 64, 96, 90, 8),
]


def test_every_launch_shape_decodes_identically(pvvc_lib, torch, gop):
    dec = pvvc_lib.Decoder(nslots=128, max_leaves=4096)
    ref = decode_batch(torch, pvvc_lib, dec, gop)
    assert (ref[2] == 0).all()
    for t in TUNES:
        out = decode_batch(torch, pvvc_lib, dec, gop, tune=t)
        for a, b in zip(ref, out):
            assert np.array_equal(a, b), t


def test_plan_info_counts(pvvc_lib, gop):
    default = pvvc_lib.Plan(gop).info()
    assert default["tune"] == {"group_ctas_per_sm": 3, "min_group": 4, "rlgr_block": 64, "rlgr_long_ctas": 16,
                               "rlgr_mid_pct": 50, "rlgr_long_lanes": 32}
    assert default["nslices"] == gop.nslices
    assert default["nintra"] == int(((gop.type & 0x02) == 0).sum())
    # every slot's intra slice heads a phase-A group; 8 frames -> its 7 P slices join it
    ones = pvvc_lib.Plan(gop, tune=(3, 32, 128, -1, -1, 32)).info()
    assert ones["groups_a"] == default["nintra"] and ones["singles_a"] == 0
    k = ones
    # trees, one per-slice RLGR launch (8-frame groups are below the windowed RLGR's 16), then the inverse-RAHT
    # launches
    assert k["kernels"] == 2 + (k["groups_a"] > 0) + (k["singles_a"] > 0) + (k["groups_b"] > 0) + (k["singles_b"] > 0)
    assert k["clear_bytes"] > 0


def test_autotune_returns_a_valid_shape(pvvc_lib, torch, gop):
    dec = pvvc_lib.Decoder(nslots=128, max_leaves=4096)
    ref = decode_batch(torch, pvvc_lib, dec, gop)
    pay = _dev(torch, gop.payload)
    stream = torch.cuda.current_stream().cuda_stream
    best, ms = pvvc_lib.autotune(gop, dec, pay.data_ptr(), reps=2, stream=stream)
    assert ms > 0
    assert best["group_ctas_per_sm"] in (1, 2, 3, 4) and best["rlgr_block"] in (32, 64, 128, 256)
    assert best["rlgr_long_ctas"] in (-1, 16, 32, 48, 64, 96) and best["rlgr_mid_pct"] in (-1, 15, 30, 50, 70)
    assert best["rlgr_long_lanes"] in (8, 16, 32)
    assert 1 <= best["min_group"] <= 32
    out = decode_batch(torch, pvvc_lib, dec, gop, tune=best)
    for a, b in zip(ref, out):
        assert np.array_equal(a, b)


def test_graph_replay_matches_direct_decode(pvvc_lib, torch, gop):
    dec = pvvc_lib.Decoder(nslots=128, max_leaves=4096)
    ref = decode_batch(torch, pvvc_lib, dec, gop, points24=True)
    plan = pvvc_lib.Plan(gop)
    P = plan.total_points
    pay = _dev(torch, gop.payload)
    xyz = torch.zeros((P, 3), dtype=torch.float32, device="cuda")
    rgb = torch.zeros((P, 3), dtype=torch.uint8, device="cuda")
    p24 = torch.zeros((P, 6), dtype=torch.float32, device="cuda")
    st = torch.full((gop.nslices,), -1, dtype=torch.int32, device="cuda")
    ws = torch.empty(plan.workspace_bytes, dtype=torch.uint8, device="cuda")
    g = plan.graph(dec, pay.data_ptr(), xyz.data_ptr(), rgb.data_ptr(), p24.data_ptr(), st.data_ptr(), ws.data_ptr(),
                   ws.numel())
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        xyz.zero_(); rgb.zero_(); p24.zero_(); st.fill_(-1)
        g.launch(stream)
        torch.cuda.synchronize()
        got = (xyz.cpu().numpy(), rgb.cpu().numpy(), st.cpu().numpy(), p24.cpu().numpy())
        for a, b in zip(ref, got):
            assert np.array_equal(a, b)
    g.close()
